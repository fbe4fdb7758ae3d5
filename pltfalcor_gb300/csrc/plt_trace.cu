// Closest-hit and any-hit BVH traversal kernels (one thread per ray, persistent grid-stride
// loop).  Replaces DXR TraceRay over the scene acceleration structure
// (RenderPasses/PLTPT/pltpt_sample.rt.slang:168-183 and ShadowRays.slangh:65-135 in
// ssteinberg/PLTFalcor).  Nodes are read as four 16-byte loads through the read-only path; the
// traversal stack (node, entry distance) lives in registers/local memory with a fixed depth bound
// checked against overflow.
#include "plt_internal.h"
#include "plt_trace.cuh"

namespace pltdev {

using plt::BvhNode;
using plt::TraceParams;

template <bool ANY>
__device__ __forceinline__ void traceOne(const TraceParams& P, uint32_t i, uint32_t& nodeVisits, uint32_t& triTests) {
    const uint32_t n = P.n;
    const float ox = __ldg(P.origin + i), oy = __ldg(P.origin + n + i), oz = __ldg(P.origin + 2 * n + i);
    const float dx = __ldg(P.dir + i), dy = __ldg(P.dir + n + i), dz = __ldg(P.dir + 2 * n + i);
    const float tmin = P.tmin ? __ldg(P.tmin + i) : 0.f;
    const float tmax = P.tmax ? __ldg(P.tmax + i) : 3.402823466e+38f;
    uint32_t overflow = 0;
    const TraceResult h = traverse<ANY>(reinterpret_cast<const float4*>(P.nodes), P.tris, ox, oy, oz, dx, dy, dz, tmin, tmax,
                                        nodeVisits, triTests, overflow, 0, P.stackCap);
    if (overflow) atomicOr(P.status, plt::kStatusStackOverflow);
    if (ANY) {
        P.occluded[i] = h.prim != 0xFFFFFFFFu ? 1u : 0u;
    } else {
        P.prim[i] = h.prim;
        if (P.t) P.t[i] = h.prim != 0xFFFFFFFFu ? h.t : -1.f;
        if (P.bary) { P.bary[i] = h.b1; P.bary[n + i] = h.b2; }
    }
}

template <bool ANY>
__global__ void __launch_bounds__(128) traceKernel(const TraceParams P) {
    uint32_t nodeVisits = 0, triTests = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < P.n; i += gridDim.x * blockDim.x) traceOne<ANY>(P, i, nodeVisits, triTests);
    if (P.stats) {
        // warp-reduce the traversal counters, one atomic per warp
        unsigned long long nv = nodeVisits, tt = triTests;
        for (int o = 16; o > 0; o >>= 1) {
            nv += __shfl_down_sync(0xFFFFFFFFu, nv, o);
            tt += __shfl_down_sync(0xFFFFFFFFu, tt, o);
        }
        if ((threadIdx.x & 31u) == 0) {
            atomicAdd(P.stats, nv);
            atomicAdd(P.stats + 1, tt);
        }
    }
}

}  // namespace pltdev

namespace plt {

cudaError_t launchTrace(const TraceParams& p, bool any, int numSMs, cudaStream_t stream) {
    if (p.n == 0) return cudaSuccess;
    static int bpsClosest = -1, bpsAny = -1;
    int& bps = any ? bpsAny : bpsClosest;
    if (bps < 0) {
        int b = 0;
        if (any) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, pltdev::traceKernel<true>, 128, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, pltdev::traceKernel<false>, 128, 0);
        bps = b > 0 ? b : 1;
    }
    uint32_t grid = (uint32_t)(numSMs * bps);
    const uint32_t need = (p.n + 127) / 128;
    if (grid > need) grid = need;
    if (any) pltdev::traceKernel<true><<<grid, 128, 0, stream>>>(p);
    else pltdev::traceKernel<false><<<grid, 128, 0, stream>>>(p);
    return cudaGetLastError();
}

}  // namespace plt
