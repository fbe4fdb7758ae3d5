// Instantiation of the fused BSDF batch kernel for 8 hero wavelength(s) per beam.
#include "plt_bsdf_kernel.cuh"

namespace plt {
template cudaError_t launchBsdfBatchH<8>(const BatchParams&, int, cudaStream_t);
}  // namespace plt
