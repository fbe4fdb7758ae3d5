// Solve pass instantiated for 8 hero wavelengths (beyond the reference's 1-4) per path.
#include "plt_pt.cuh"

namespace pltdev {
template <> cudaError_t launchSolveH<8>(const PtParams& p, const plt::PtLaunch& L, int numSMs, cudaStream_t stream) {
    return launchSolve<8>(p, L, numSMs, stream);
}
}  // namespace pltdev
