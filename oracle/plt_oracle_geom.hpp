// ORACLE -- test infrastructure only.  Geometry helpers of the path-tracing oracle, restated from
// ssteinberg/PLTFalcor (citations per function), compiled with FP contraction off:
//   intersectRayTriangle   Source/Falcor/Utils/Geometry/IntersectionHelpers.slang:102-166
//   computeRayOrigin       Source/Falcor/Utils/Geometry/GeometryHelpers.slang:47-60
//   oct (equal-area) maps  Source/Falcor/Utils/Math/MathHelpers.slang:147-243
//   snorm16 packing        Source/Falcor/Utils/Math/FormatConversion.slang:216-258,
//                          Source/Falcor/Utils/Math/PackedFormats.slang:50-62
//   sample_triangle        Source/Falcor/Utils/Math/MathHelpers.slang:372-377
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <algorithm>
#include <vector>

namespace plt_oracle {
namespace geom {

inline bool intersectRayTriangle(const float o[3], const float d[3], const float* v, float& t, float& b1, float& b2) {
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

// Brute force over tri[ntri][9]: closest hit in [t0, t1] (ties to the lowest index), or the first
// hit when `any`.  Returns the primitive or 0xFFFFFFFF.
inline uint32_t traceBrute(const float* tri, uint32_t ntri, const float o[3], const float d[3], float t0, float t1, bool any,
                           float& tHit, float& b1, float& b2) {
    float bestT = t1, bb1 = 0.f, bb2 = 0.f;
    uint32_t best = 0xFFFFFFFFu;
    for (uint32_t k = 0; k < ntri; ++k) {
        float t, u, v;
        if (!intersectRayTriangle(o, d, tri + 9 * (size_t)k, t, u, v)) continue;
        if (!(t >= t0) || !(t <= bestT)) continue;
        if (t < bestT || k < best) {
            bestT = t;
            best = k;
            bb1 = u;
            bb2 = v;
            if (any) break;
        }
    }
    tHit = bestT;
    b1 = bb1;
    b2 = bb2;
    return best;
}

inline int32_t f2i(float f) { int32_t i; std::memcpy(&i, &f, 4); return i; }
inline float i2f(int32_t i) { float f; std::memcpy(&f, &i, 4); return f; }

// computeRayOrigin: integer-ulp offset away from the surface, GeometryHelpers.slang:47-60
inline void computeRayOrigin(const float pos[3], const float n[3], float out[3]) {
    const float origin = 1.f / 16.f;
    const float fScale = 3.f / 65536.f;
    const float iScale = 3 * 256.f;
    for (int c = 0; c < 3; ++c) {
        const int32_t iOff = (int32_t)(n[c] * iScale);
        const float iPos = i2f(f2i(pos[c]) + (pos[c] < 0.f ? -iOff : iOff));
        const float fOff = n[c] * fScale;
        out[c] = std::fabs(pos[c]) < origin ? pos[c] + fOff : iPos;
    }
}

inline float hsign(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }

// ndir_to_oct_equal_area_snorm / oct_to_ndir_equal_area_snorm, MathHelpers.slang:199-243
inline void ndirToOctEqualArea(const float n[3], float p[2]) {
    const float r = std::sqrt(1.f - std::fabs(n[2]));
    const float phi = std::atan2(std::fabs(n[1]), std::fabs(n[0]));
    float py = r * phi * 0.636619772367581343076f;   // M_2_PI
    float px = r - py;
    if (n[2] < 0.f) {
        const float tx = 1.f - py, ty = 1.f - px;
        px = tx;
        py = ty;
    }
    p[0] = px * hsign(n[0]);
    p[1] = py * hsign(n[1]);
}
inline void octToNdirEqualArea(const float p[2], float n[3]) {
    const float d = 1.f - (std::fabs(p[0]) + std::fabs(p[1]));
    const float r = 1.f - std::fabs(d);
    const float phi = (r > 0.f) ? ((std::fabs(p[1]) - std::fabs(p[0])) / r + 1.f) * 0.785398163397448309616f : 0.f;  // M_PI_4
    const float f = r * std::sqrt(2.f - r * r);
    n[0] = f * hsign(p[0]) * std::cos(phi);
    n[1] = f * hsign(p[1]) * std::sin(phi);
    n[2] = hsign(d) * (1.f - r * r);
}

// ndir_to_oct_snorm / oct_to_ndir_snorm (non equal-area), MathHelpers.slang:147-185
inline void octWrap(float& x, float& y) {
    const float nx = (1.f - std::fabs(y)) * (x >= 0.f ? 1.f : -1.f);
    const float ny = (1.f - std::fabs(x)) * (y >= 0.f ? 1.f : -1.f);
    x = nx;
    y = ny;
}
inline int32_t floatToSnorm16(float v) {
    v = std::isnan(v) ? 0.f : std::fmin(std::fmax(v, -1.f), 1.f);
    return (int32_t)std::trunc(v * 32767.f + (v >= 0.f ? 0.5f : -0.5f));
}
// encodeNormal2x16 -> decodeNormal2x16 round trip (the emissive-triangle normal as the reference
// stores it, LightCollectionShared.slang:82-126)
inline void quantizeNormal2x16(const float n[3], float out[3]) {
    const float s = 1.f / (std::fabs(n[0]) + std::fabs(n[1]) + std::fabs(n[2]));
    float px = n[0] * s, py = n[1] * s;
    if (n[2] < 0.f) octWrap(px, py);
    const uint32_t packed = ((uint32_t)floatToSnorm16(px) & 0xFFFFu) | ((uint32_t)floatToSnorm16(py) << 16);
    const int32_t bx = (int32_t)(packed << 16) >> 16, by = (int32_t)packed >> 16;
    const float ux = std::fmax((float)bx / 32767.f, -1.f), uy = std::fmax((float)by / 32767.f, -1.f);
    float x = ux, y = uy, z = 1.f - std::fabs(ux) - std::fabs(uy);
    if (z < 0.f) octWrap(x, y);
    const float l = std::sqrt(x * x + y * y + z * z);
    out[0] = x / l;
    out[1] = y / l;
    out[2] = z / l;
}

// float -> binary16 bits, round to nearest even (finite inputs in the half range)
inline uint16_t floatToHalfRne(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const int32_t e = (int32_t)((x >> 23) & 0xFF) - 127 + 15;
    uint32_t m = x & 0x7FFFFFu;
    if (((x >> 23) & 0xFF) == 0xFF) return (uint16_t)(sign | 0x7C00u | (m ? 0x200u : 0u));
    if (e >= 31) return (uint16_t)(sign | 0x7C00u);
    if (e <= 0) {
        if (e < -10) return (uint16_t)sign;
        m |= 0x800000u;
        const int shift = 14 - e;
        uint32_t hm = m >> shift;
        const uint32_t rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (hm & 1u))) ++hm;
        return (uint16_t)(sign | hm);
    }
    uint32_t h = ((uint32_t)e << 10) | (m >> 13);
    const uint32_t rem = m & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
}


// Bounding-volume hierarchy over tri[ntri][9] for the oracle's ray casts: median splits on the
// longest centroid axis, up to 4 triangles per leaf, boxes padded by 2^-18 of their extent plus
// 2^-20 of the coordinate magnitude so no box that holds a hit can be culled.  The query returns
// exactly what traceBrute returns (lowest t in [t0, t1], ties to the lowest index).
struct OracleBvh {
    struct Node { float lo[3], hi[3]; int32_t left, right, first, count; };
    std::vector<Node> nodes;
    std::vector<uint32_t> order;
    const float* tri = nullptr;

    void build(const float* t, uint32_t n) {
        tri = t;
        order.resize(n);
        for (uint32_t i = 0; i < n; ++i) order[i] = i;
        nodes.clear();
        nodes.reserve(2 * (size_t)n + 1);
        if (n) buildRec(0, n);
    }
    int32_t buildRec(uint32_t b, uint32_t e) {
        Node nd;
        for (int c = 0; c < 3; ++c) { nd.lo[c] = INFINITY; nd.hi[c] = -INFINITY; }
        float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (uint32_t i = b; i < e; ++i) {
            const float* v = tri + 9 * (size_t)order[i];
            for (int c = 0; c < 3; ++c) {
                const float mn = std::fmin(v[c], std::fmin(v[3 + c], v[6 + c]));
                const float mx = std::fmax(v[c], std::fmax(v[3 + c], v[6 + c]));
                nd.lo[c] = std::fmin(nd.lo[c], mn);
                nd.hi[c] = std::fmax(nd.hi[c], mx);
                const float ce = 0.5f * (mn + mx);
                clo[c] = std::fmin(clo[c], ce);
                chi[c] = std::fmax(chi[c], ce);
            }
        }
        for (int c = 0; c < 3; ++c) {
            const float pad = (nd.hi[c] - nd.lo[c]) * 0x1p-18f + std::fmax(std::fabs(nd.lo[c]), std::fabs(nd.hi[c])) * 0x1p-20f + 1e-30f;
            nd.lo[c] -= pad;
            nd.hi[c] += pad;
        }
        const int32_t id = (int32_t)nodes.size();
        nodes.push_back(nd);
        if (e - b <= 4) {
            nodes[id].left = nodes[id].right = -1;
            nodes[id].first = (int32_t)b;
            nodes[id].count = (int32_t)(e - b);
            return id;
        }
        int axis = 0;
        for (int c = 1; c < 3; ++c) if (chi[c] - clo[c] > chi[axis] - clo[axis]) axis = c;
        const uint32_t mid = b + (e - b) / 2;
        auto key = [&](uint32_t t) {
            const float* v = tri + 9 * (size_t)t;
            return std::fmin(v[axis], std::fmin(v[3 + axis], v[6 + axis])) + std::fmax(v[axis], std::fmax(v[3 + axis], v[6 + axis]));
        };
        std::nth_element(order.begin() + b, order.begin() + mid, order.begin() + e,
                         [&](uint32_t x, uint32_t y) { const float kx = key(x), ky = key(y); return kx < ky || (kx == ky && x < y); });
        const int32_t l = buildRec(b, mid);
        const int32_t r = buildRec(mid, e);
        nodes[id].left = l;
        nodes[id].right = r;
        nodes[id].first = nodes[id].count = 0;
        return id;
    }
    static bool slab(const Node& n, const float o[3], const float inv[3], float t0, float t1) {
        float tn = t0, tf = t1;
        for (int c = 0; c < 3; ++c) {
            float a = (n.lo[c] - o[c]) * inv[c], b = (n.hi[c] - o[c]) * inv[c];
            if (std::isnan(a) || std::isnan(b)) { a = -INFINITY; b = INFINITY; }
            if (a > b) std::swap(a, b);
            tn = std::fmax(tn, a);
            tf = std::fmin(tf, b);
        }
        return tn <= tf * 1.0000005f;
    }
    uint32_t trace(const float o[3], const float d[3], float t0, float t1, bool any, float& tHit, float& b1, float& b2) const {
        float bestT = t1, bb1 = 0.f, bb2 = 0.f;
        uint32_t best = 0xFFFFFFFFu;
        tHit = bestT;
        b1 = b2 = 0.f;
        const float dsum = std::fabs(d[0]) + std::fabs(d[1]) + std::fabs(d[2]);
        if (nodes.empty() || !(dsum > 0.f) || !(dsum < INFINITY)) return best;
        const float inv[3] = {1.f / d[0], 1.f / d[1], 1.f / d[2]};
        int32_t stack[128];
        int sp = 0;
        stack[sp++] = 0;
        while (sp > 0) {
            const Node& n = nodes[(size_t)stack[--sp]];
            if (!slab(n, o, inv, t0 - std::fabs(t0) * 1e-6f, bestT)) continue;
            if (n.left < 0) {
                for (int32_t i = n.first; i < n.first + n.count; ++i) {
                    const uint32_t k = order[(size_t)i];
                    float t, u, v;
                    if (!intersectRayTriangle(o, d, tri + 9 * (size_t)k, t, u, v)) continue;
                    if (!(t >= t0) || !(t <= bestT)) continue;
                    if (t < bestT || k < best) {
                        bestT = t;
                        best = k;
                        bb1 = u;
                        bb2 = v;
                        if (any) { tHit = bestT; b1 = bb1; b2 = bb2; return best; }
                    }
                }
            } else {
                if (sp + 2 > 128) return traceFallback(o, d, t0, t1, any, tHit, b1, b2);
                stack[sp++] = n.right;
                stack[sp++] = n.left;
            }
        }
        tHit = bestT;
        b1 = bb1;
        b2 = bb2;
        return best;
    }
    uint32_t traceFallback(const float o[3], const float d[3], float t0, float t1, bool any, float& tHit, float& b1, float& b2) const {
        return traceBrute(tri, (uint32_t)order.size(), o, d, t0, t1, any, tHit, b1, b2);
    }
};

}  // namespace geom
}  // namespace plt_oracle
