// Solve pass instantiated for 1 hero wavelength(s) per path.
#include "plt_pt.cuh"

namespace pltdev {
template <> cudaError_t launchSolveH<1>(const PtParams& p, const plt::PtLaunch& L, int numSMs, cudaStream_t stream) {
    return launchSolve<1>(p, L, numSMs, stream);
}
}  // namespace pltdev
