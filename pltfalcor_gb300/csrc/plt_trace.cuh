// BVH traversal on sm_103a (GB300 has no RT cores): closest-hit and any-hit queries against the
// host-built SAH BVH.  Intersection is the reference's watertight ray/triangle test
// (Source/Falcor/Utils/Geometry/IntersectionHelpers.slang:102-166 in ssteinberg/PLTFalcor), written
// with explicitly rounded operations (__fmul_rn etc. are never contracted into FMAs) so hits,
// distances and barycentrics are bit-identical to a CPU evaluation of the same expressions.
// Ties at equal distance resolve to the lowest primitive index, the brute-force oracle's rule.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "plt_bvh.h"

namespace pltdev {

struct TriHit {
    float t, b1, b2;   // distance, barycentrics of vertices 1 and 2
    bool hit;
};

// The ray-only part of intersectRayTriangle: the dominant axis kz, the other two (swapped for a
// negative direction along kz) and the shear constants.  The same for every triangle of a ray.
struct WtRay {
    int kx, ky, kz;
    float Sx, Sy, Sz;
};
__device__ __forceinline__ WtRay wtRay(float dx, float dy, float dz) {
    WtRay r;
    const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
    int kz = 0;
    if (ay > ax && ay > az) kz = 1;
    if (az > ax && az > ay) kz = 2;
    int kx = kz + 1 == 3 ? 0 : kz + 1;
    int ky = kx + 1 == 3 ? 0 : kx + 1;
    const float dkz = kz == 0 ? dx : (kz == 1 ? dy : dz);
    if (dkz < 0.f) { const int s = kx; kx = ky; ky = s; }
    const float dkx = kx == 0 ? dx : (kx == 1 ? dy : dz);
    const float dky = ky == 0 ? dx : (ky == 1 ? dy : dz);
    r.kx = kx;
    r.ky = ky;
    r.kz = kz;
    r.Sx = __fdiv_rn(dkx, dkz);
    r.Sy = __fdiv_rn(dky, dkz);
    r.Sz = __fdiv_rn(1.f, dkz);
    return r;
}

// intersectRayTriangle with a rounding-exact evaluation; A = v0 - o etc.
__device__ __forceinline__ TriHit watertight(float ox, float oy, float oz, const WtRay& R, float4 v0, float4 v1, float4 v2) {
    TriHit h;
    h.hit = false;
    const int kx = R.kx, ky = R.ky, kz = R.kz;
    const float Sx = R.Sx, Sy = R.Sy, Sz = R.Sz;
    const float A[3] = {__fsub_rn(v0.x, ox), __fsub_rn(v0.y, oy), __fsub_rn(v0.z, oz)};
    const float B[3] = {__fsub_rn(v1.x, ox), __fsub_rn(v1.y, oy), __fsub_rn(v1.z, oz)};
    const float C[3] = {__fsub_rn(v2.x, ox), __fsub_rn(v2.y, oy), __fsub_rn(v2.z, oz)};
    auto pick = [](const float* v, int k) { return k == 0 ? v[0] : (k == 1 ? v[1] : v[2]); };
    const float Akz = pick(A, kz), Bkz = pick(B, kz), Ckz = pick(C, kz);
    const float Ax = __fsub_rn(pick(A, kx), __fmul_rn(Sx, Akz));
    const float Ay = __fsub_rn(pick(A, ky), __fmul_rn(Sy, Akz));
    const float Bx = __fsub_rn(pick(B, kx), __fmul_rn(Sx, Bkz));
    const float By = __fsub_rn(pick(B, ky), __fmul_rn(Sy, Bkz));
    const float Cx = __fsub_rn(pick(C, kx), __fmul_rn(Sx, Ckz));
    const float Cy = __fsub_rn(pick(C, ky), __fmul_rn(Sy, Ckz));
    float U = __fsub_rn(__fmul_rn(Cx, By), __fmul_rn(Cy, Bx));
    float V = __fsub_rn(__fmul_rn(Ax, Cy), __fmul_rn(Ay, Cx));
    float W = __fsub_rn(__fmul_rn(Bx, Ay), __fmul_rn(By, Ax));
    if (U == 0.f || V == 0.f || W == 0.f) {
        U = (float)__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx));
        V = (float)__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx));
        W = (float)__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax));
    }
    if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return h;
    const float det = __fadd_rn(__fadd_rn(U, V), W);
    if (det == 0.f) return h;
    const float Az = __fmul_rn(Sz, Akz), Bz = __fmul_rn(Sz, Bkz), Cz = __fmul_rn(Sz, Ckz);
    const float T = __fadd_rn(__fadd_rn(__fmul_rn(U, Az), __fmul_rn(V, Bz)), __fmul_rn(W, Cz));
    const float rcp = __fdiv_rn(1.f, det);
    h.t = __fmul_rn(T, rcp);
    h.b1 = __fmul_rn(V, rcp);
    h.b2 = __fmul_rn(W, rcp);
    h.hit = true;
    return h;
}

// Robust culling margin: computed slab distances carry up to ~2 ulp of relative error (Ize, "Robust
// BVH Ray Traversal", JCGT 2013: exit * (1 + 2 gamma_3)); a box is culled only when its computed
// entry exceeds a distance times this factor.  The same factor guards the stack-pop test against
// the current closest hit, so a box whose face holds the hit point is never dropped.
constexpr float kTfarScale = 1.000000477f;  // 1 + 2^-21 > 1 + 2 gamma_3 (gamma_3 = 3 u / (1 - 3 u), u = 2^-24)

// Conservative slab test: entry/exit with the exit widened by kTfarScale.
__device__ __forceinline__ bool slab(const float* mn, const float* mx, float ox, float oy, float oz, float ix, float iy, float iz,
                                     float tmin, float tmax, float& tenter) {
    const float tx0 = (mn[0] - ox) * ix, tx1 = (mx[0] - ox) * ix;
    const float ty0 = (mn[1] - oy) * iy, ty1 = (mx[1] - oy) * iy;
    const float tz0 = (mn[2] - oz) * iz, tz1 = (mx[2] - oz) * iz;
    const float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin));
    const float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax)) * kTfarScale;
    tenter = tn;
    return tn <= tf;
}

constexpr int kStackDepth = 64;

__device__ __forceinline__ float safeRcp(float d) { return d != 0.f ? __fdiv_rn(1.f, d) : copysignf(INFINITY, d); }

// Result of one BVH query.
struct TraceResult {
    uint32_t prim;      // triangle id, 0xFFFFFFFF on a miss
    float t, b1, b2;
};

// ---- traversal state and steps; dynamic fetch (Aila & Laine, "Understanding the Efficiency of Ray
// Traversal on GPUs", HPG 2009) -------------------------------------------------------------------
// One lane's ray in flight: its traversal state between steps.  Any visit order finds the same
// closest hit: boxes are culled only beyond the current closest distance (with the kTfarScale
// margin) and equal distances resolve to the lowest triangle id.
constexpr int32_t kTravDone = -2147483647 - 1;   // `node` of a ray that cannot hit anything

struct TravLane {
    float ox, oy, oz, ix, iy, iz, tmin, bestT, bestB1, bestB2;
    uint32_t bestPrim;
    WtRay wr;
    int32_t node;
    int sp;   // entries on the lane's stack (kept apart from this struct, so its scalars stay in registers)

    __device__ __forceinline__ void start(float px, float py, float pz, float dx, float dy, float dz, float t0, float t1, int32_t root) {
        ox = px;
        oy = py;
        oz = pz;
        tmin = t0;
        bestT = t1;
        bestB1 = bestB2 = 0.f;
        bestPrim = 0xFFFFFFFFu;
        sp = 0;
        node = root;
        // a zero or non-finite direction cannot hit anything (see traverse)
        const float dsum = fabsf(dx) + fabsf(dy) + fabsf(dz);
        if (!(dsum > 0.f) || !(dsum < INFINITY)) node = kTravDone;
        ix = safeRcp(dx);
        iy = safeRcp(dy);
        iz = safeRcp(dz);
        wr = wtRay(dx, dy, dz);
    }

    // The nearest pending node (inner or leaf) that can still hold a closer hit, or kTravDone.
    __device__ __forceinline__ int32_t pop(const int2* stack) {
        while (sp > 0) {
            const int2 e = stack[--sp];
            if (__int_as_float(e.y) <= bestT * kTfarScale) return e.x;
        }
        return kTravDone;
    }

    // Tests the triangles of leaf `ref`; true when an any-hit query has found its hit.
    template <bool ANY>
    __device__ __forceinline__ bool testLeaf(const float4* __restrict__ tris, int32_t ref, uint32_t& triTests) {
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
                return true;
            }
            if (th.t < bestT || prim < bestPrim) {
                bestT = th.t;
                bestPrim = prim;
                bestB1 = th.b1;
                bestB2 = th.b2;
            }
        }
        return false;
    }

    // One step in while-while form with speculative leaf postponement (Aila & Laine 2009): inner
    // nodes are visited until every lane of the warp holds a leaf to test (a lane that reaches a
    // leaf first keeps it and goes on with the next inner node), then each lane tests its leaves.
    // Leaves are nodes of the traversal order here (pushed and popped like inner nodes); the closest
    // hit found is the same.  True when the ray has finished.
    template <bool ANY>
    __device__ __forceinline__ bool stepWW(const float4* __restrict__ nodes, const float4* __restrict__ tris, int2* stack, int stackCap,
                                           uint32_t& nodeVisits, uint32_t& triTests, uint32_t& overflow) {
        int32_t leaf = 0;   // the postponed leaf (a negative reference), 0: none
        while (node >= 0) {
            ++nodeVisits;
            const float4 a = __ldg(nodes + 4 * node), b = __ldg(nodes + 4 * node + 1), c = __ldg(nodes + 4 * node + 2);
            const int4 rr = __ldg(reinterpret_cast<const int4*>(nodes) + 4 * node + 3);
            const float lmn[3] = {a.x, a.y, a.z}, lmx[3] = {a.w, b.x, b.y};
            const float rmn[3] = {b.z, b.w, c.x}, rmx[3] = {c.y, c.z, c.w};
            float tl = 0.f, tr = 0.f;
            const bool hl = rr.x != plt::kNoChild && slab(lmn, lmx, ox, oy, oz, ix, iy, iz, tmin, bestT, tl);
            const bool hr = rr.y != plt::kNoChild && slab(rmn, rmx, ox, oy, oz, ix, iy, iz, tmin, bestT, tr);
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
                node = pop(stack);
            }
            if (node < 0 && node != kTravDone && leaf == 0) {
                leaf = node;
                node = pop(stack);
            }
            if (!__any_sync(__activemask(), leaf == 0)) break;
        }
        while (leaf < 0) {
            if (testLeaf<ANY>(tris, leaf, triTests)) return true;
            leaf = 0;
            if (node < 0 && node != kTravDone) {
                leaf = node;
                node = pop(stack);
            }
        }
        return node == kTravDone;
    }
};

// Stack traversal of the two-wide BVH for one ray: closest hit with tmin <= t <= tmax (ties to
// the lowest triangle id), or, with ANY, the first hit found (TraceRay with
// ACCEPT_FIRST_HIT_AND_END_SEARCH).  The ray's lane runs while-while steps (TravLane::stepWW) until
// it has finished, so the lanes of a warp tracing together test their leaves together.  Counts node
// visits and triangle tests; sets `overflow` when the fixed-depth stack (or the caller's smaller
// cap, stackCap) overflowed: the result is then possibly not the closest.
template <bool ANY>
__device__ __forceinline__ TraceResult traverse(const float4* __restrict__ nodes, const float4* __restrict__ tris, float ox, float oy,
                                                float oz, float dx, float dy, float dz, float tmin, float tmax,
                                                uint32_t& nodeVisits, uint32_t& triTests, uint32_t& overflow, int32_t root = 0,
                                                int stackCap = kStackDepth) {
    TravLane L;
    L.start(ox, oy, oz, dx, dy, dz, tmin, tmax, root);
    int2 stack[kStackDepth];
    while (!L.template stepWW<ANY>(nodes, tris, stack, stackCap, nodeVisits, triTests, overflow)) {
    }
    TraceResult res;
    res.prim = L.bestPrim;
    res.t = L.bestT;
    res.b1 = L.bestB1;
    res.b2 = L.bestB2;
    return res;
}

// Lanes of a warp whose ray has finished take new rays together once at least this many are idle
// (or the whole warp is).  Measured on 2^20 random closest-hit rays of a 1.04 M-triangle scene
// (rays/s) with one node visit per step: 1 lane 1.36 G, 4 1.46 G, 8 1.47 G, 16 1.43 G, 32 1.18 G
// (1024^2 primary rays 1.68, 2.07, 2.22, 2.20, 2.33 G); with while-while steps (stepWW): 4 lanes
// 2.00 G, 8 2.00 G, 16 2.00 G (primary 2.79, 2.89, 3.06 G).
#ifndef PLT_TRACE_REFILL
#define PLT_TRACE_REFILL 16
#endif

// A ray handed to dynamicTraversal: origin, direction, [tmin, tmax] and the BVH root.
struct TravRay {
    float ox, oy, oz, dx, dy, dz, tmin, tmax;
    int32_t root;
};

// Traces rays [begin, end) with one ray per lane and dynamic fetch: every loop iteration is one
// while-while step (TravLane::stepWW) per active lane; a lane whose ray r has finished calls finish(r, prim, t, b1, b2) and goes
// idle, and idle lanes are refilled together (fetch(r) returns ray r's TravRay) from the shared
// counter `next` (initialised to begin by the caller, then a __syncthreads), so a warp keeps its
// lanes busy instead of waiting for the longest ray of a fixed set of 32.  Whole warps only.
template <bool ANY, class Fetch, class Finish>
__device__ __forceinline__ void dynamicTraversal(const float4* __restrict__ nodes, const float4* __restrict__ tris, int stackCap, uint32_t end,
                                                 uint32_t* next, Fetch fetch, Finish finish, uint32_t& nodeVisits, uint32_t& triTests,
                                                 uint32_t& overflow) {
    constexpr uint32_t kNoRay = 0xFFFFFFFFu, kFull = 0xFFFFFFFFu;
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t ray = kNoRay;
    bool drained = false;
    TravLane L;
    L.node = kTravDone;
    int2 stack[kStackDepth];
    for (;;) {
        const unsigned idle = __ballot_sync(kFull, ray == kNoRay);
        if (idle == kFull && drained) break;
        if (!drained && (idle == kFull || __popc(idle) >= PLT_TRACE_REFILL)) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(next, (uint32_t)__popc(idle));
            base = __shfl_sync(kFull, base, 0);
            if (base >= end) drained = true;
            if (ray == kNoRay) {
                const uint32_t r = base + (uint32_t)__popc(idle & ((1u << lane) - 1u));
                if (r < end) {
                    ray = r;
                    const TravRay q = fetch(r);
                    L.start(q.ox, q.oy, q.oz, q.dx, q.dy, q.dz, q.tmin, q.tmax, q.root);
                }
            }
        }
        if (ray == kNoRay) continue;
        if (L.template stepWW<ANY>(nodes, tris, stack, stackCap, nodeVisits, triTests, overflow)) {
            finish(ray, L.bestPrim, L.bestT, L.bestB1, L.bestB2);
            ray = kNoRay;
        }
    }
}

}  // namespace pltdev
