// ORACLE -- test infrastructure only.  Brute-force closest-hit / any-hit over all triangles with the
// reference's watertight ray/triangle test, restated from
// Source/Falcor/Utils/Geometry/IntersectionHelpers.slang:102-166 (ssteinberg/PLTFalcor), compiled
// with FP contraction off.  Closest hit: lowest t with tmin <= t <= tmax, ties to the lowest index.
#include <cmath>
#include <cstdint>
#include <cstring>

namespace {

bool intersectRayTriangle(const float o[3], const float d[3], const float* v, float& t, float& b1, float& b2) {
    const float absDir[3] = {std::fabs(d[0]), std::fabs(d[1]), std::fabs(d[2])};
    unsigned axis = 0;
    if (absDir[1] > absDir[0] && absDir[1] > absDir[2]) axis = 1;
    if (absDir[2] > absDir[0] && absDir[2] > absDir[1]) axis = 2;
    unsigned kz = axis;
    unsigned kx = (kz + 1) % 3;
    unsigned ky = (kx + 1) % 3;
    if (d[kz] < 0.f) { const unsigned s = kx; kx = ky; ky = s; }
    const float Sx = d[kx] / d[kz];
    const float Sy = d[ky] / d[kz];
    const float Sz = 1.f / d[kz];
    const float A[3] = {v[0] - o[0], v[1] - o[1], v[2] - o[2]};
    const float B[3] = {v[3] - o[0], v[4] - o[1], v[5] - o[2]};
    const float C[3] = {v[6] - o[0], v[7] - o[1], v[8] - o[2]};
    const float Ax = A[kx] - Sx * A[kz];
    const float Ay = A[ky] - Sy * A[kz];
    const float Bx = B[kx] - Sx * B[kz];
    const float By = B[ky] - Sy * B[kz];
    const float Cx = C[kx] - Sx * C[kz];
    const float Cy = C[ky] - Sy * C[kz];
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.f || V == 0.f || W == 0.f) {
        const double CxBy = (double)Cx * (double)By, CyBx = (double)Cy * (double)Bx;
        U = (float)(CxBy - CyBx);
        const double AxCy = (double)Ax * (double)Cy, AyCx = (double)Ay * (double)Cx;
        V = (float)(AxCy - AyCx);
        const double BxAy = (double)Bx * (double)Ay, ByAx = (double)By * (double)Ax;
        W = (float)(BxAy - ByAx);
    }
    if ((U < 0.f || V < 0.f || W < 0.f) && (U > 0.f || V > 0.f || W > 0.f)) return false;
    const float det = U + V + W;
    if (det == 0.f) return false;
    const float Az = Sz * A[kz];
    const float Bz = Sz * B[kz];
    const float Cz = Sz * C[kz];
    const float T = U * Az + V * Bz + W * Cz;
    const float rcpDet = 1.f / det;
    t = T * rcpDet;
    b1 = V * rcpDet;
    b2 = W * rcpDet;
    return true;
}

}  // namespace

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

}  // extern "C"
