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

constexpr int kStackDepth = 64;

__device__ __forceinline__ float safeRcp(float d) { return d != 0.f ? __fdiv_rn(1.f, d) : copysignf(INFINITY, d); }

template <bool ANY>
__device__ __forceinline__ void traceOne(const TraceParams& P, uint32_t i, uint32_t& nodeVisits, uint32_t& triTests) {
    const uint32_t n = P.n;
    const float ox = __ldg(P.origin + i), oy = __ldg(P.origin + n + i), oz = __ldg(P.origin + 2 * n + i);
    const float dx = __ldg(P.dir + i), dy = __ldg(P.dir + n + i), dz = __ldg(P.dir + 2 * n + i);
    const float tmin = P.tmin ? __ldg(P.tmin + i) : 0.f;
    const float tmax = P.tmax ? __ldg(P.tmax + i) : 3.402823466e+38f;
    const float ix = safeRcp(dx), iy = safeRcp(dy), iz = safeRcp(dz);
    const float4* __restrict__ nodes = reinterpret_cast<const float4*>(P.nodes);
    const float4* __restrict__ tris = P.tris;

    float bestT = tmax, bestB1 = 0.f, bestB2 = 0.f;
    uint32_t bestPrim = 0xFFFFFFFFu;
    bool done = false;
    int2 stack[kStackDepth];
    int sp = 0;
    int32_t node = 0;
    uint32_t overflow = 0;

    auto leaf = [&](int32_t ref) {
        const uint32_t v = (uint32_t)~ref;
        const uint32_t first = v >> 4, count = (v & 15u) + 1u;
        for (uint32_t k = first; k < first + count; ++k) {
            const float4 v0 = __ldg(tris + 3 * k), v1 = __ldg(tris + 3 * k + 1), v2 = __ldg(tris + 3 * k + 2);
            ++triTests;
            const TriHit h = watertight(ox, oy, oz, dx, dy, dz, v0, v1, v2);
            if (!h.hit || !(h.t >= tmin) || !(h.t <= bestT)) continue;
            const uint32_t prim = __float_as_uint(v0.w);
            if (ANY) {
                bestT = h.t;
                bestPrim = prim;
                done = true;
                return;
            }
            if (h.t < bestT || prim < bestPrim) {
                bestT = h.t;
                bestPrim = prim;
                bestB1 = h.b1;
                bestB2 = h.b2;
            }
        }
    };

    for (;;) {
        ++nodeVisits;
        const float4 a = __ldg(nodes + 4 * node), b = __ldg(nodes + 4 * node + 1), c = __ldg(nodes + 4 * node + 2);
        const int4 r = __ldg(reinterpret_cast<const int4*>(nodes) + 4 * node + 3);
        const float lmn[3] = {a.x, a.y, a.z}, lmx[3] = {a.w, b.x, b.y};
        const float rmn[3] = {b.z, b.w, c.x}, rmx[3] = {c.y, c.z, c.w};
        float tl = 0.f, tr = 0.f;
        bool hl = r.x != plt::kNoChild && slab(lmn, lmx, ox, oy, oz, ix, iy, iz, tmin, bestT, tl);
        bool hr = r.y != plt::kNoChild && slab(rmn, rmx, ox, oy, oz, ix, iy, iz, tmin, bestT, tr);
        if (hl && r.x < 0) { leaf(r.x); hl = false; if (ANY && done) break; }
        if (hr && r.y < 0) { leaf(r.y); hr = false; if (ANY && done) break; }
        if (hl && hr) {
            const bool leftNear = tl <= tr;
            if (sp < kStackDepth) stack[sp++] = make_int2(leftNear ? r.y : r.x, __float_as_int(leftNear ? tr : tl));
            else overflow = 1;
            node = leftNear ? r.x : r.y;
            continue;
        }
        if (hl) { node = r.x; continue; }
        if (hr) { node = r.y; continue; }
        // pop the nearest pending node that can still hold a closer hit
        bool found = false;
        while (sp > 0) {
            const int2 e = stack[--sp];
            if (__int_as_float(e.y) <= bestT * kTfarScale) { node = e.x; found = true; break; }
        }
        if (!found) break;
    }
    if (overflow) atomicOr(P.status, plt::kStatusStackOverflow);
    if (ANY) {
        P.occluded[i] = bestPrim != 0xFFFFFFFFu ? 1u : 0u;
    } else {
        P.prim[i] = bestPrim;
        if (P.t) P.t[i] = bestPrim != 0xFFFFFFFFu ? bestT : -1.f;
        if (P.bary) { P.bary[i] = bestB1; P.bary[n + i] = bestB2; }
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
