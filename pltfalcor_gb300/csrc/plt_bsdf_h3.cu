// Instantiation of the fused BSDF batch kernel for 3 hero wavelength(s) per beam.
#include "plt_bsdf_kernel.cuh"

namespace plt {
template cudaError_t launchBsdfBatchH<3>(const BatchParams&, int, cudaStream_t);
}  // namespace plt
