// ORACLE -- test infrastructure only.  Brute-force closest-hit / any-hit over all triangles with the
// reference's watertight ray/triangle test, restated from
// Source/Falcor/Utils/Geometry/IntersectionHelpers.slang:102-166 (ssteinberg/PLTFalcor), compiled
// with FP contraction off.  Closest hit: lowest t with tmin <= t <= tmax, ties to the lowest index.
#include <cmath>
#include <cstdint>
#include <cstring>

#include "plt_oracle_geom.hpp"

using plt_oracle::geom::intersectRayTriangle;

extern "C" {

// tri: [ntri][9] vertex coordinates; rays SoA planes [3][n]; tmin/tmax may be NULL.
// any = 0: prim/t/bary (closest); any = 1: occluded.
void plto_trace_brute(const float* tri, uint32_t ntri, const float* origin, const float* dir, const float* tmin,
                      const float* tmax, uint32_t n, int any, uint32_t* prim, float* tout, float* bary, uint32_t* occluded,
                      int threads) {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1) if (threads != 1)
#endif
    for (long long ii = 0; ii < (long long)n; ++ii) {
        const uint32_t i = (uint32_t)ii;
        const float o[3] = {origin[i], origin[n + i], origin[2 * (size_t)n + i]};
        const float d[3] = {dir[i], dir[n + i], dir[2 * (size_t)n + i]};
        const float t0 = tmin ? tmin[i] : 0.f;
        const float t1 = tmax ? tmax[i] : 3.402823466e+38f;
        float bestT = t1, bb1 = 0.f, bb2 = 0.f;
        uint32_t best = 0xFFFFFFFFu;
        for (uint32_t k = 0; k < ntri; ++k) {
            float t, b1, b2;
            if (!intersectRayTriangle(o, d, tri + 9 * (size_t)k, t, b1, b2)) continue;
            if (!(t >= t0) || !(t <= bestT)) continue;
            if (t < bestT || k < best) {
                bestT = t;
                best = k;
                bb1 = b1;
                bb2 = b2;
                if (any) break;
            }
        }
        if (any) {
            occluded[i] = best != 0xFFFFFFFFu ? 1u : 0u;
        } else {
            prim[i] = best;
            if (tout) tout[i] = best != 0xFFFFFFFFu ? bestT : -1.f;
            if (bary) { bary[i] = bb1; bary[n + i] = bb2; }
        }
    }
}

// Same query through the oracle's own BVH (plt_oracle_geom.hpp); must return what the brute force
// returns (hit ids, distances, barycentrics) -- the path-tracing oracle casts its rays this way.
void plto_trace_bvh(const float* tri, uint32_t ntri, const float* origin, const float* dir, const float* tmin,
                    const float* tmax, uint32_t n, int any, uint32_t* prim, float* tout, float* bary, uint32_t* occluded,
                    int threads) {
    plt_oracle::geom::OracleBvh bvh;
    bvh.build(tri, ntri);
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(threads > 0 ? threads : 1) if (threads != 1)
#endif
    for (long long ii = 0; ii < (long long)n; ++ii) {
        const uint32_t i = (uint32_t)ii;
        const float o[3] = {origin[i], origin[n + i], origin[2 * (size_t)n + i]};
        const float d[3] = {dir[i], dir[n + i], dir[2 * (size_t)n + i]};
        const float t0 = tmin ? tmin[i] : 0.f;
        const float t1 = tmax ? tmax[i] : 3.402823466e+38f;
        float t, b1, b2;
        const uint32_t best = bvh.trace(o, d, t0, t1, any != 0, t, b1, b2);
        if (any) {
            occluded[i] = best != 0xFFFFFFFFu ? 1u : 0u;
        } else {
            prim[i] = best;
            if (tout) tout[i] = best != 0xFFFFFFFFu ? t : -1.f;
            if (bary) { bary[i] = b1; bary[n + i] = b2; }
        }
    }
}

}  // extern "C"
