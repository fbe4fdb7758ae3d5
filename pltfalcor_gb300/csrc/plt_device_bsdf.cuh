// Device PLT BSDFs (sm_103a) behind the batched IMaterialInstance ABI.
//
// Reference (paths inside ssteinberg/PLTFalcor): Rendering/PLT.slang:41-245 (beam),
// Rendering/Materials/PLT/{GaussianSurface,FractalSurface,DiffractionGrating,Interference,
// Birefringence}.slang and the PLT*BSDF.slang BxDFs / IMaterialInstance wrappers, with material
// decode from PLT*Material.slang.  Layout and arithmetic are GPU-first: one thread per query,
// material constants precomputed once per material on the host (DevMaterial), Fresnel Mueller
// products in 4-parameter block form, frame rotations without trigonometric round trips.
#pragma once

#include "plt_device_math.cuh"
#include "plt_layout.h"

namespace pltdev {

constexpr uint32_t kMatDiffuse = 2, kMatConductor = 3, kMatDielectric = 4, kMatOpaqueDielectric = 5, kMatThin = 6,
                   kMatCoatedConductor = 7, kMatCoatedOpaque = 8, kMatGratedConductor = 9, kMatGratedOpaque = 10,
                   kMatMultilayer = 11, kMatTypeCount = 12;

// mean wavenumber 2*pi/(550e-3 um) (FractalSurface.slang:43)
__device__ __forceinline__ float meank() { return k2Pi / (550.0f * 1e-3f); }

struct Ctx {
    const DevProfile* profiles;   // shared-memory copy of the spectral profiles
    uint32_t nprof;
    uint32_t flags;               // PLT_OPTION_* bits
};

// ------------------------------------------------------------------------------------------
// Beam (PLT.slang:83-245) for H hero wavelengths
// ------------------------------------------------------------------------------------------
template <int H> struct DBeam {
    float L[4][H];
    float wl[H];
    float D0, D1, D2, r_m;
    f3 r, t;

    PLT_DI f4 getSP(int j) const { return f4{L[0][j], L[1][j], L[2][j], L[3][j]}; }
    PLT_DI void setSP(int j, f4 s) { L[0][j] = s.x; L[1][j] = s.y; L[2][j] = s.z; L[3][j] = s.w; }
    PLT_DI void setZero() {
#pragma unroll
        for (int j = 0; j < H; ++j) L[0][j] = L[1][j] = L[2][j] = L[3][j] = 0.f;
    }
    PLT_DI float rmm() const { return r_m * 1e+3f; }
    PLT_DI f3 toLocal(f3 v) const { return mk3(dot(v, t), dot(v, cross(t, r)), dot(v, r)); }
    // transformCoherence: D <- U^T D U (PLT.slang:73-77)
    PLT_DI void transformCoherence(float u00, float u01, float u10, float u11) {
        const float a00 = D0 * u00 + D1 * u10, a01 = D0 * u01 + D1 * u11;
        const float a10 = D1 * u00 + D2 * u10, a11 = D1 * u01 + D2 * u11;
        const float n00 = u00 * a00 + u10 * a10;
        const float n01 = u00 * a01 + u10 * a11;
        const float n11 = u01 * a01 + u11 * a11;
        D0 = n00; D1 = n01; D2 = n11;
    }
    // rotateFrame with MuellerT (PLT.slang:203-216, Mueller.slang:34-53): sin/cos of
    // theta = atan2(y, x) are taken directly as y/|(x,y)| and x/|(x,y)|.
    PLT_DI void rotateFrame(f3 newt, f3 newr) {
        const float y = dot(r, cross(t, newt));
        const float x = dot(t, newt);
        const float h = sqrtf(x * x + y * y);
        float s = 0.f, c = 1.f;
        if (h > 0.f && h < INFINITY) { s = y / h; c = x / h; }
        const float rx = 2.f * s * c;
        const float ry = 1.f - 2.f * s * s;
#pragma unroll
        for (int j = 0; j < H; ++j) {
            const float s1 = L[1][j], s2 = L[2][j];
            L[1][j] = rx * s1 - ry * s2;
            L[2][j] = ry * s1 + rx * s2;
        }
        transformCoherence(c, -s, s, c);
        r = newr;
        t = newt;
    }
    PLT_DI void constructLocalFrame(f3 wo) { rotateFrame(canonical_tangent(wo), wo); }
    // Q() (PLT.slang:146-150): [[t.x, b.x], [t.y, b.y]], b = cross(t, r)
    // mutualCoherence (hwss k), PLT.slang:164-169
    PLT_DI float coherenceQuad(f3 v) const {
        const float s = sqr(1.f / rmm());
        const float i00 = s * D0, i01 = s * D1, i11 = s * D2;
        return v.x * (i00 * v.x + i01 * v.y) + v.y * (i01 * v.x + i11 * v.y);
    }
    PLT_DI float mutualCoherenceK(float k, float quad) const { return expf(-.5f * (sqr(k / k2Pi) * quad)); }
    // mutualCoherenceAngular, PLT.slang:172-177
    PLT_DI float mutualCoherenceAngular(f3 d1, f3 d2) const {
        const float s4 = 3.5449077018110318f;  // sqrt(4 pi)
        const float vx = 1.f / fmaxf(s4 * fabsf(d1.x - d2.x), kFltEps);
        const float vy = 1.f / fmaxf(s4 * fabsf(d1.y - d2.y), kFltEps);
        const float rm = rmm();
        const float s = sqr(1.f / rm), s2 = sqr(rm);
        const float i00 = s * D0 * s2, i01 = s * D1 * s2, i11 = s * D2 * s2;
        const float x = 1.f / (vx * (i00 * vx + i01 * vy) + vy * (i01 * vx + i11 * vy));
        return expf(-.5f * x);
    }
};

PLT_DI float kOfWl(float wl) { return k2Pi / (1e-3f * wl); }
PLT_DI f3 reflectL(f3 w) { return mk3(-w.x, -w.y, w.z); }
PLT_DI float m00Of(const float* __restrict__ tab, float wl) { return __ldg(tab + spectrumBin(wl)); }

// ------------------------------------------------------------------------------------------
// Gaussian surface (GaussianSurface.slang:37-110)
// ------------------------------------------------------------------------------------------
// Specular fraction alpha = exp(-x) together with 1 - alpha.  The shaders form 1 - alpha by
// subtraction, which loses every digit as alpha -> 1 (smooth surfaces, grazing gratings); here
// it is -expm1(-x), accurate to an ulp.  Discrete choices (u < alpha) use alpha itself.
struct Alpha { float a, om; };
PLT_DI Alpha alphaOf(float x) { return Alpha{expf(-x), -expm1f(-x)}; }
PLT_DI Alpha gaussAlpha(const float* __restrict__ p, f3 wi, f3 wo, float k) {
    const float q = __ldg(p + PG_Q);
    const float x = sqr((fabsf(wi.z) + fabsf(wo.z)) * q * k);
    return q == 0.f ? Alpha{1.f, 0.f} : alphaOf(x);
}
// sample_boxmueller_truncated (MathHelpers.slang:416-434)
PLT_DI f2 boxMullerTruncated(float u0, float u1, f2 mean, float sigma2, float& pdf) {
    const float mm = dot(mean, mean);
    const float l = sqrtf(fminf(1.f, mm));
    const float coso = sqrtf(fmaxf(0.f, 1.f - mm));
    const float phi_i = (mean.x != 0.f || mean.y != 0.f) ? atan2f(mean.y, mean.x) : 0.f;
    const float s = expf(-.5f * sqr(1.f + l) / sigma2);
    const float x = (1.f - s) * fmaxf(kFltEps, u0) + s;
    const float r = sqrtf(-2.f * sigma2 * logf(x));
    const float max_phi = (r < kFltEps || l < kFltEps) ? kPi : acosf(clampf((r * r + l * l - 1.f) / (2.f * r * l), -1.f, 1.f));
    const float phi = phi_i + kPi + max_phi * (2.f * u1 - 1.f);
    float sp, cp;
    sincosf(phi, &sp, &cp);
    pdf = .5f * x / (max_phi * sigma2) * coso;
    return f2{r * cp + mean.x, r * sp + mean.y};
}
PLT_NI float boxMullerTruncatedPdf(f2 wo, f2 mean, float sigma2) {
    const float mm = dot(mean, mean);
    const float l = sqrtf(fminf(1.f, mm));
    const float coso = sqrtf(fmaxf(0.f, 1.f - mm));
    const f2 d = f2{wo.x - mean.x, wo.y - mean.y};
    const float r2 = dot(d, d);
    const float x = expf(-.5f * r2 / sigma2);
    const float r = sqrtf(r2);
    const float max_phi = (r < kFltEps || l < kFltEps) ? kPi : acosf(clampf((r * r + l * l - 1.f) / (2.f * r * l), -1.f, 1.f));
    return .5f * x / (max_phi * sigma2) * coso;
}
// uw: when uw.x >= 0, the primary sample (u0, u1) of the direction is replaced by uw after the
// generator has drawn its own pair (a primary-sample-space warp; the generator's stream is unchanged).
PLT_NI f3 gaussSample(const float* __restrict__ p, f3 wi, SampleGen& sg, float k, float& pdf, f2 uw) {
    const float s2 = __ldg(p + PG_INVSIGMA2) / (k * k);
    float u0 = sg.next1D(), u1 = sg.next1D();
    if (uw.x >= 0.f) { u0 = uw.x; u1 = uw.y; }
    const f2 wo = boxMullerTruncated(u0, u1, f2{-wi.x, -wi.y}, s2, pdf);
    const float z = sqrtf(fmaxf(0.f, 1.f - dot(wo, wo)));
    return mk3(wo.x, wo.y, signf(wi.z) * z);
}
PLT_DI float gaussPdf(const float* __restrict__ p, f3 wi, f3 wo, float k) {
    const float s2 = __ldg(p + PG_INVSIGMA2) / (k * k);
    return boxMullerTruncatedPdf(f2{wo.x, wo.y}, f2{-wi.x, -wi.y}, s2);
}
// eval(k, invTheta(1), Q, h): S = I/sigma2 + Q invTheta Q^T
template <int H>
PLT_DI float gaussEval(const float* __restrict__ p, const DBeam<H>& b, float k, f3 h) {
    // invTheta(1) = sqr((1/2pi)/r_mm) * D
    const float sc = sqr((1.f / k2Pi) / b.rmm());
    const float t00 = sc * b.D0, t01 = sc * b.D1, t11 = sc * b.D2;
    const f3 bb = cross(b.t, b.r);
    const float q00 = b.t.x, q01 = bb.x, q10 = b.t.y, q11 = bb.y;
    // Q * invTheta * Q^T
    const float a00 = t00 * q00 + t01 * q01, a01 = t00 * q10 + t01 * q11;   // invTheta * Q^T
    const float a10 = t01 * q00 + t11 * q01, a11 = t01 * q10 + t11 * q11;
    const float is2 = __ldg(p + PG_INVSIGMA2);
    const float s00 = is2 + (q00 * a00 + q01 * a10);
    const float s01 = 0.f + (q00 * a01 + q01 * a11);
    const float s10 = 0.f + (q10 * a00 + q11 * a10);
    const float s11 = is2 + (q10 * a01 + q11 * a11);
    const float d = s00 * s11 - s01 * s10;
    const float i00 = s11 / d, i01 = -s01 / d, i10 = -s10 / d, i11 = s00 / d;
    const float quad = h.x * (i00 * h.x + i01 * h.y) + h.y * (i10 * h.x + i11 * h.y);
    return expf(-.5f * (k * k) * quad) * ((k * k) * k1_2Pi / sqrtf(d));
}

// ------------------------------------------------------------------------------------------
// Fractal (K-correlation / ABC) surface (FractalSurface.slang:38-135)
// ------------------------------------------------------------------------------------------
PLT_DI Alpha fracAlpha(const float* __restrict__ p, f3 wi, f3 wo, float k) {
    return alphaOf(sqr((fabsf(wi.z) + fabsf(wo.z)) * __ldg(p + PF_Q) * k));
}
PLT_NI float fracPGF(const float* __restrict__ p, float zx, float zy) {
    const float f = 1.f / powPos(1.f + __ldg(p + PF_T) * (zx * zx + zy * zy), __ldg(p + PF_EXPO));
    return __ldg(p + PF_C) * f;
}
PLT_NI f3 fracSample(const float* __restrict__ p, f3 wi, SampleGen& sg, float k, float& pdf, f2 uw) {
    const float s = sqrtf(fmaxf(0.f, 1.f - wi.z * wi.z));
    const float phi_i = s > 0.f ? atan2f(wi.y, wi.x) : 0.f;
    const float T = __ldg(p + PF_T);
    float u0 = sg.next1D(), u1 = sg.next1D();
    if (uw.x >= 0.f) { u0 = uw.x; u1 = uw.y; }
    sg.next(); sg.next();  // FractalSurface.sample draws a second, unused 2D sample
    const float M = 1.f - powf(1.f + k * k * T * sqr(1.f + s), __ldg(p + PF_SEXP));
    const float f = sqrtf(powf(1.f - M * u0, __ldg(p + PF_IEXP)) - 1.f) / __ldg(p + PF_SQRTT);
    const float fk = f / k;
    const float phi_max = (f == 0.f || s == 0.f) ? kPi : acosf(clampf((fk * fk + s * s - 1.f) / (2.f * fk * s), -1.f, 1.f));
    const float phi_f = phi_i + (2.f * u1 - 1.f) * phi_max;
    float sf, cf;
    sincosf(phi_f, &sf, &cf);
    const float vx = f * cf, vy = f * sf;
    const float wx = vx / k - wi.x, wy = vy / k - wi.y;
    const float z = sqrtf(fmaxf(0.f, 1.f - (wx * wx + wy * wy)));
    pdf = kPi / phi_max * z * fracPGF(p, vx, vy);
    return mk3(wx, wy, signf(wi.z) * z);
}
PLT_DI float fracPdf(const float* __restrict__ p, f3 wi, f3 wo, float k) { return fracPGF(p, k * (wi.x + wo.x), k * (wi.y + wo.y)); }

// ------------------------------------------------------------------------------------------
// Interference (Interference.slang:36-57)
// ------------------------------------------------------------------------------------------
// sqrt(max(0, x y)) as sqrt|x| sqrt|y|: the product of two intensities of ~1e-20 is subnormal,
// which the BSDF batch units flush to zero, while the split form keeps its cross term.
PLT_DI float geoMean(float x, float y) {
    return ((x > 0.f && y > 0.f) || (x < 0.f && y < 0.f)) ? sqrtf(fabsf(x)) * sqrtf(fabsf(y)) : 0.f;
}
PLT_DI f4 interfere(f4 a, f4 b, float ps, float pp, float coh) {
    const float S1 = (a.x + a.y) / 2.f, P1 = (a.x - a.y) / 2.f;
    const float S2 = (b.x + b.y) / 2.f, P2 = (b.x - b.y) / 2.f;
    const float S = S1 + S2 + 2.f * geoMean(S1, S2) * ps * coh;
    const float P = P1 + P2 + 2.f * geoMean(P1, P2) * pp * coh;
    const float n = a.x + b.x > 1e-6f ? (S + P) / (a.x + b.x) : 0.f;
    return f4{S + P, S - P, (a.z + b.z) * n, (a.w + b.w) * n};
}

// result of one query
template <int H> struct QOut {
    float pdf;
    float lpdf[H];
    f3 sWo;
    float sPdf, sWeight;
    uint32_t sLobe, sValid;
};

// scatter-lobe coherence transform diag(c, 1/c), c = sqrt(max(1e-2, |wo.z|))
template <int H> PLT_DI void scatterCoherence(DBeam<H>& b, f3 wo, bool isDirect) {
    if (isDirect) { b.transformCoherence(1.f, 0.f, 0.f, 1.f); return; }
    const float c = sqrtf(fmaxf(1e-2f, fabsf(wo.z)));
    b.transformCoherence(c, 0.f, 0.f, 1.f / c);
}

}  // namespace pltdev

#include "plt_device_materials.cuh"
