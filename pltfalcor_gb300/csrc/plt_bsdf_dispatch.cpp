// Hero-wavelength dispatch of the fused BSDF batch kernel (one instantiation per translation unit).
#include "plt_internal.h"

namespace plt {

template <int H>
cudaError_t launchBsdfBatchH(const BatchParams& p, int numSMs, cudaStream_t stream);

cudaError_t launchBsdfBatch(const BatchParams& p, int hwss, int numSMs, cudaStream_t stream) {
    switch (hwss) {
    case 1: return launchBsdfBatchH<1>(p, numSMs, stream);
    case 2: return launchBsdfBatchH<2>(p, numSMs, stream);
    case 3: return launchBsdfBatchH<3>(p, numSMs, stream);
    case 4: return launchBsdfBatchH<4>(p, numSMs, stream);
    case 8: return launchBsdfBatchH<8>(p, numSMs, stream);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace plt
