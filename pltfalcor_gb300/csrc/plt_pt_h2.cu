// Solve pass instantiated for 2 hero wavelength(s) per path.
#include "plt_pt.cuh"

namespace pltdev {
template <> cudaError_t launchSolveH<2>(const PtParams& p, const plt::PtLaunch& L, int numSMs, cudaStream_t stream) {
    return launchSolve<2>(p, L, numSMs, stream);
}
}  // namespace pltdev
