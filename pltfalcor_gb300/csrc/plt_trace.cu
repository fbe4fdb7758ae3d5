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

// Lanes of a warp whose ray has finished take new rays together once at least this many are idle
// (or the whole warp is), from the CTA's range of rays through a shared-memory counter.
#ifndef PLT_TRACE_REFILL
#define PLT_TRACE_REFILL 8
#endif

// One ray per lane with dynamic fetch (Aila & Laine, "Understanding the Efficiency of Ray Traversal
// on GPUs", HPG 2009): each loop iteration visits one node per active lane (and tests the triangles
// of the leaves it hits); a lane whose ray has finished writes its result and goes idle, and idle
// lanes are refilled from the CTA's contiguous share of the rays, so a warp keeps its lanes busy
// instead of waiting for the longest ray of a fixed set of 32.  The traversal order of each ray is
// that of traverse() (plt_trace.cuh), so hits are identical.
template <bool ANY>
__global__ void __launch_bounds__(128) traceKernel(const TraceParams P) {
    constexpr uint32_t kNoRay = 0xFFFFFFFFu, kFull = 0xFFFFFFFFu;
    __shared__ uint32_t next;
    const uint32_t per = (P.n + gridDim.x - 1) / gridDim.x;
    const uint32_t begin = min(blockIdx.x * per, P.n), end = min(begin + per, P.n);
    if (threadIdx.x == 0) next = begin;
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t n = P.n;
    const float4* __restrict__ nodes = reinterpret_cast<const float4*>(P.nodes);
    const float4* __restrict__ tris = P.tris;
    const int stackCap = P.stackCap;
    uint32_t nodeVisits = 0, triTests = 0, overflow = 0;
    uint32_t ray = kNoRay;
    bool drained = false;
    float ox = 0.f, oy = 0.f, oz = 0.f, ix = 0.f, iy = 0.f, iz = 0.f, tmin = 0.f;
    float bestT = 0.f, bestB1 = 0.f, bestB2 = 0.f;
    uint32_t bestPrim = 0xFFFFFFFFu;
    WtRay wr{0, 1, 2, 0.f, 0.f, 0.f};
    int32_t node = 0;
    int sp = 0;
    int2 stack[kStackDepth];
    for (;;) {
        const unsigned idle = __ballot_sync(kFull, ray == kNoRay);
        if (idle == kFull && drained) break;
        if (!drained && (idle == kFull || __popc(idle) >= PLT_TRACE_REFILL)) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(&next, (uint32_t)__popc(idle));
            base = __shfl_sync(kFull, base, 0);
            if (base >= end) drained = true;
            if (ray == kNoRay) {
                const uint32_t r = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (r < end) {
                    ray = r;
                    ox = __ldg(P.origin + r);
                    oy = __ldg(P.origin + n + r);
                    oz = __ldg(P.origin + 2 * n + r);
                    const float dx = __ldg(P.dir + r), dy = __ldg(P.dir + n + r), dz = __ldg(P.dir + 2 * n + r);
                    tmin = P.tmin ? __ldg(P.tmin + r) : 0.f;
                    bestT = P.tmax ? __ldg(P.tmax + r) : 3.402823466e+38f;
                    bestB1 = bestB2 = 0.f;
                    bestPrim = 0xFFFFFFFFu;
                    node = 0;
                    sp = 0;
                    // a zero or non-finite direction cannot hit anything (see traverse)
                    const float dsum = fabsf(dx) + fabsf(dy) + fabsf(dz);
                    if (!(dsum > 0.f) || !(dsum < INFINITY)) node = -1 - (int32_t)0x7FFFFFFF;   // finished below
                    ix = safeRcp(dx);
                    iy = safeRcp(dy);
                    iz = safeRcp(dz);
                    wr = wtRay(dx, dy, dz);
                }
            }
        }
        if (ray == kNoRay) continue;
        bool finished = node == -1 - (int32_t)0x7FFFFFFF;
        if (!finished) {
            ++nodeVisits;
            const float4 a = __ldg(nodes + 4 * node), b = __ldg(nodes + 4 * node + 1), c = __ldg(nodes + 4 * node + 2);
            const int4 rr = __ldg(reinterpret_cast<const int4*>(nodes) + 4 * node + 3);
            const float lmn[3] = {a.x, a.y, a.z}, lmx[3] = {a.w, b.x, b.y};
            const float rmn[3] = {b.z, b.w, c.x}, rmx[3] = {c.y, c.z, c.w};
            float tl = 0.f, tr = 0.f;
            bool hl = rr.x != plt::kNoChild && slab(lmn, lmx, ox, oy, oz, ix, iy, iz, tmin, bestT, tl);
            bool hr = rr.y != plt::kNoChild && slab(rmn, rmx, ox, oy, oz, ix, iy, iz, tmin, bestT, tr);
#pragma unroll
            for (int side = 0; side < 2; ++side) {
                const bool h = side ? hr : hl;
                const int32_t ref = side ? rr.y : rr.x;
                if (!h || ref >= 0 || finished) continue;
                if (side) hr = false;
                else hl = false;
                const uint32_t v = (uint32_t)~ref;
                const uint32_t first = v >> 4, count = (v & 15u) + 1u;
                for (uint32_t k = first; k < first + count; ++k) {
                    const float4 v0 = __ldg(tris + 3 * k), v1 = __ldg(tris + 3 * k + 1), v2 = __ldg(tris + 3 * k + 2);
                    ++triTests;
                    const TriHit th = watertight(ox, oy, oz, wr, v0, v1, v2);
                    if (!th.hit || !(th.t >= tmin) || !(th.t <= bestT)) continue;
                    const uint32_t prim = __float_as_uint(v0.w);
                    if (ANY) {
                        bestT = th.t;
                        bestPrim = prim;
                        finished = true;
                        break;
                    }
                    if (th.t < bestT || prim < bestPrim) {
                        bestT = th.t;
                        bestPrim = prim;
                        bestB1 = th.b1;
                        bestB2 = th.b2;
                    }
                }
            }
            if (!finished) {
                if (hl && hr) {
                    const bool leftNear = tl <= tr;
                    if (sp < stackCap && sp < kStackDepth) stack[sp++] = make_int2(leftNear ? rr.y : rr.x, __float_as_int(leftNear ? tr : tl));
                    else overflow = 1;
                    node = leftNear ? rr.x : rr.y;
                } else if (hl) {
                    node = rr.x;
                } else if (hr) {
                    node = rr.y;
                } else {
                    // pop the nearest pending node that can still hold a closer hit
                    finished = true;
                    while (sp > 0) {
                        const int2 e = stack[--sp];
                        if (__int_as_float(e.y) <= bestT * kTfarScale) {
                            node = e.x;
                            finished = false;
                            break;
                        }
                    }
                }
            }
        }
        if (finished) {
            if (ANY) {
                P.occluded[ray] = bestPrim != 0xFFFFFFFFu ? 1u : 0u;
            } else {
                P.prim[ray] = bestPrim;
                if (P.t) P.t[ray] = bestPrim != 0xFFFFFFFFu ? bestT : -1.f;
                if (P.bary) {
                    P.bary[ray] = bestB1;
                    P.bary[n + ray] = bestB2;
                }
            }
            ray = kNoRay;
        }
    }
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
