// Solve pass instantiated for 4 hero wavelength(s) per path.
#include "plt_pt.cuh"

namespace pltdev {
template <> cudaError_t launchSolveH<4>(const PtParams& p, int numSMs, cudaStream_t stream) { return launchSolve<4>(p, numSMs, stream); }
}  // namespace pltdev
