// plt_bsdf_batch_noalloc: the batched BSDF entry point for callers that must not allocate device
// memory.  plt_bsdf_batch sorts every batch through a scratch buffer (a per-tile permutation and a
// work counter) that the context grows with cudaMalloc on first use of a larger batch; this variant
// uses the file-scope device array below instead, so it never calls cudaMalloc or cudaFree.
//
// The array is a module global: every GPU that loads the library holds its
// kNoAllocScratchBytes (about 2 MB) until the process exits, whether or not the entry point is used.
// Host code cannot use the array's name as a device address (it names a host-side stand-in), so
// the first call on each device resolves the address with cudaGetSymbolAddress while that device
// is current and caches it; that first call should happen before any stream capture begins.
// All calls on a device share the array, so two calls whose work overlaps on the GPU race on it:
// serialise them (one stream, or events).  Nothing in it needs clearing between calls: the
// classify kernel rewrites the whole permutation and tile ranges it uses, and the schedule's
// counters, which must be zero when a batch starts, are zero in the freshly loaded array and are
// zeroed again by every batch once it has read them.  The call runs on the context's device only (PLT_INVALID_ARG when
// another device is current), so the address it uses is always that device's copy of the array.
// A cudaDeviceReset unloads the library's device code and invalidates every context of that
// device together with the cached address: do not call this entry point after one in the same
// process.
#include <cuda_runtime.h>

#include <mutex>

#include "plt_internal.h"

namespace {

constexpr uint32_t kNoAllocMaxQueries = PLT_NOALLOC_MAX_QUERIES;
constexpr size_t kNoAllocScratchBytes = plt::bsdfScratchBytes(kNoAllocMaxQueries);
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocScratchBytes];

std::mutex g_addrMutex;
void* g_addr[kMaxDevices] = {};

// Device address of g_noallocScratch on the current device (set-up on first use per device).
cudaError_t scratchAddress(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_addrMutex);
    if (!g_addr[dev]) {
        void* a = nullptr;
        e = cudaGetSymbolAddress(&a, g_noallocScratch);
        if (e != cudaSuccess) return e;
        g_addr[dev] = a;
    }
    *out = g_addr[dev];
    return cudaSuccess;
}

}  // namespace

extern "C" plt_status plt_bsdf_batch_noalloc(plt_context* ctx, const plt_bsdf_queries* q, const plt_bsdf_results* r,
                                             uint32_t ops, void* stream) {
    if (!q) return PLT_INVALID_ARG;
    if (q->n > kNoAllocMaxQueries) return PLT_TOO_LARGE;
    plt::BatchParams p{};
    int numSMs = 0;
    const plt_status s = plt::fillBatchParams(ctx, q, r, ops, &p, &numSMs);
    if (s != PLT_OK || q->n == 0) return s;
    void* base = nullptr;
    if (scratchAddress(&base) != cudaSuccess) return PLT_CUDA_ERROR;
    plt::pltBatchScratch(p, base);
    const cudaError_t e = plt::launchBsdfBatch(p, (int)q->hwss, numSMs, (cudaStream_t)stream);
    return e == cudaSuccess ? PLT_OK : PLT_CUDA_ERROR;
}
