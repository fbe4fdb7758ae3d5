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

// One ray per lane with dynamic fetch (dynamicTraversal, plt_trace.cuh): each CTA traces a
// contiguous share of the rays, its warps refilling idle lanes from a shared-memory counter.  56
// registers (9 CTAs per SM); bounding it to 10 CTAs measured the same, to 12 (40 registers, spills)
// 29 % slower.
template <bool ANY>
__global__ void __launch_bounds__(128) traceKernel(const TraceParams P) {
    __shared__ uint32_t next;
    const uint32_t n = P.n;
    const uint32_t per = (n + gridDim.x - 1) / gridDim.x;
    const uint32_t begin = min(blockIdx.x * per, n), end = min(begin + per, n);
    if (threadIdx.x == 0) next = begin;
    __syncthreads();
    uint32_t nodeVisits = 0, triTests = 0, overflow = 0;
    dynamicTraversal<ANY>(
        reinterpret_cast<const float4*>(P.nodes), P.tris, P.stackCap, end, &next,
        [&](uint32_t r) {
            return TravRay{__ldg(P.origin + r), __ldg(P.origin + n + r), __ldg(P.origin + 2 * n + r), __ldg(P.dir + r), __ldg(P.dir + n + r),
                           __ldg(P.dir + 2 * n + r), P.tmin ? __ldg(P.tmin + r) : 0.f, P.tmax ? __ldg(P.tmax + r) : 3.402823466e+38f, 0};
        },
        [&](uint32_t r, uint32_t prim, float t, float b1, float b2) {
            if (ANY) {
                P.occluded[r] = prim != 0xFFFFFFFFu ? 1u : 0u;
            } else {
                P.prim[r] = prim;
                if (P.t) P.t[r] = prim != 0xFFFFFFFFu ? t : -1.f;
                if (P.bary) {
                    P.bary[r] = b1;
                    P.bary[n + r] = b2;
                }
            }
        },
        nodeVisits, triTests, overflow);
    if (overflow) atomicOr(P.status, plt::kStatusStackOverflow);
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
