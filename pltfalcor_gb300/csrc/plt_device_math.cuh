// Device math for the PLT BSDF kernels (sm_103a): vectors, complex numbers, Fresnel, the
// block-structured Fresnel Mueller matrices, spectra and the sample generator.
//
// Semantics follow the reference shader library (paths inside ssteinberg/PLTFalcor):
//   Utils/Math/MathHelpers.slang (complex :822-837, tryInvert :484-498, perp_stark :609-623,
//   BesselJ :851-885, truncated Box-Muller :416-450, concentric sampling :305-338),
//   Rendering/Materials/Fresnel.slang:30-90, Rendering/Materials/PLT/Mueller.slang:34-144,
//   Utils/Color/SpectrumUtils.slang:106-198, Scene/Scene.slang:251-294,
//   Utils/Sampling/{UniformSampleGenerator,SampleGeneratorInterface}.slang,
//   Utils/Sampling/Pseudorandom/{SplitMix64,Xoshiro}.slang, Utils/Math/BitTricks.slang:45-65.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/plt_gb300.h"

namespace pltdev {

#define PLT_DI __device__ __forceinline__
// Large helpers with many call sites (Fresnel, pGF, surface sampling, BesselJ, grating lobes,
// spectra): PLT_OUTLINE_HELPERS=1 emits them once and calls them (smaller code), the default
// inlines them (measured faster on GB300).
#ifndef PLT_OUTLINE_HELPERS
#define PLT_OUTLINE_HELPERS 0
#endif
#if PLT_OUTLINE_HELPERS
#define PLT_NI static __device__ __noinline__
#else
#define PLT_NI __device__ __forceinline__
#endif

constexpr float kPi = 3.14159265358979323846f;
constexpr float k2Pi = 6.28318530717958647693f;
constexpr float k4Pi = 12.5663706143591729539f;
constexpr float k1_Pi = 0.318309886183790671538f;
constexpr float k1_2Pi = 0.159154943091895335769f;
constexpr float kFltEps = 1.192092896e-07f;
constexpr uint32_t kNoProfile = 0xFFFFFFFFu;

// ---- lobe flags (Rendering/Materials/LobeType.slang:36-69) ----
constexpr uint32_t kLobeDiffuseR = 0x01u, kLobeScatterR = 0x02u, kLobeDeltaR = 0x04u, kLobeDispDeltaR = 0x08u,
                   kLobeScatterT = 0x20u, kLobeDeltaT = 0x40u, kLobeDispDeltaT = 0x80u, kLobeDelta = 0xCCu,
                   kLobeNonDelta = 0x33u, kLobeReflection = 0x0Fu, kLobeTransmission = 0xF0u, kLobeAll = 0xFFFFu,
                   kLobeMaterialSpecific = 0xFF00u;

// ---- small vector helpers ----
struct f2 { float x, y; };
// "no primary-sample warp" for the surface samplers (x < 0)
constexpr f2 kNoWarp = {-1.f, 0.f};
struct f3 { float x, y, z; };
struct f4 { float x, y, z, w; };
PLT_DI f3 mk3(float x, float y, float z) { return {x, y, z}; }
PLT_DI f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
PLT_DI f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
PLT_DI f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
PLT_DI f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
PLT_DI f3 operator/(f3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
PLT_DI float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
PLT_DI float dot(f2 a, f2 b) { return a.x * b.x + a.y * b.y; }
PLT_DI f3 cross(f3 a, f3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
PLT_DI f3 normalize(f3 a) { return a / sqrtf(dot(a, a)); }
PLT_DI float sqr(float x) { return x * x; }
// x^y for x > 0 as exp2(y log2 x) on the SFU (relative error ~1e-6 for |y log2 x| < 64), used where
// Sine and cosine of a phase of up to a few thousand radians: Cody-Waite additive reduction by
// 2 pi (split into the float nearest 2 pi and the remainder, 2 pi - 6.28318548f), then sincosf on
// [-pi, pi].  Where sincosf is the SFU approximation its error grows with |x| without the
// reduction (the multilayer recursion's phases reach ~100 rad).
PLT_DI void sincosReduced(float x, float* s, float* c) {
    const float k = rintf(x * 0.159154943091895336f);
    float r = fmaf(-k, 6.28318548202514648f, x);
    r = fmaf(-k, -1.74845553e-7f, r);
    sincosf(r, s, c);
}

// the reference calls pow on positive bases; PLT_FAST_POW=0 keeps the correctly rounded powf.
#ifndef PLT_FAST_POW
#define PLT_FAST_POW 1
#endif
PLT_DI float powPos(float x, float y) {
#if PLT_FAST_POW
    return exp2f(y * __log2f(x));
#else
    return powf(x, y);
#endif
}
PLT_DI float signf(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }
PLT_DI float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }
PLT_DI float lerpf(float a, float b, float t) { return a + (b - a) * t; }
PLT_DI f4 operator*(float s, f4 a) { return {s * a.x, s * a.y, s * a.z, s * a.w}; }

// complex numbers as f2
PLT_DI f2 cmul(f2 a, f2 b) { return {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x}; }
PLT_DI float cnorm2(f2 z) { return z.x * z.x + z.y * z.y; }
// complex quotients keep correct rounding: they feed the conductor Fresnel and resonant recursions
PLT_DI f2 cdiv(f2 a, f2 b) {
    const float n = cnorm2(b);
    const f2 c = cmul(a, f2{b.x, -b.y});
    return {__fdiv_rn(c.x, n), __fdiv_rn(c.y, n)};
}
PLT_DI f2 csqrt(f2 z) {
    const float r = sqrtf(cnorm2(z));
    const float a = sqrtf(fmaxf(0.f, r + z.x) / 2.f);
    const float b = sqrtf(fmaxf(0.f, r - z.x) / 2.f);
    return {a, signf(z.y) * b};
}

// perp_stark (MathHelpers.slang:609-623)
PLT_NI f3 perp_stark(f3 u) {
    const float ax = fabsf(u.x), ay = fabsf(u.y), az = fabsf(u.z);
    const uint32_t uyx = (ax - ay) < 0.f, uzx = (ax - az) < 0.f, uzy = (ay - az) < 0.f;
    const uint32_t xm = uyx & uzx, ym = (1u ^ xm) & uzy, zm = 1u ^ (xm | ym);
    return normalize(cross(u, mk3((float)xm, (float)ym, (float)zm)));
}
// canonical beam tangent of a direction (PLTBeam.constructLocalFrame, PLT.slang:218-223)
PLT_DI f3 canonical_tangent(f3 r) {
    const f3 t = mk3(-r.y, r.x, 0.f);  // cross((0,0,1), r)
    const float l2 = t.x * t.x + t.y * t.y;
    return l2 > 1e-8f ? t / sqrtf(l2) : perp_stark(r);
}

// ---- Fresnel (Fresnel.slang:30-90) ----
struct FresnelD { float rs, rp, ts, tp, cosT; };
PLT_NI FresnelD fresnel_dielectric(float cosI_, float eta) {
    FresnelD f;
    if (eta == 1.f) {
        f.cosT = -cosI_;
        f.rs = f.rp = 0.f;
        f.ts = f.tp = 1.f;
        return f;
    }
    eta = cosI_ > 0.f ? eta : 1.f / eta;
    const float cosI = fabsf(cosI_);
    const float cosTSqr = 1.f - (1.f - cosI * cosI) / (eta * eta);
    float cosT = sqrtf(fmaxf(0.f, cosTSqr));
    // correctly rounded quotients: at total internal reflection (cosT = 0) rs = rp = x / x must be
    // exactly 1 so that 1 - F vanishes as in the reference
    f.rs = __fdiv_rn(cosI - eta * cosT, cosI + eta * cosT);
    f.rp = __fdiv_rn(eta * cosI - cosT, eta * cosI + cosT);
    const float imp = sqrtf(eta * cosT / cosI);
    f.ts = imp * (f.rs + 1.f);
    f.tp = imp * (f.rp + 1.f) / eta;
    f.cosT = cosT * (-signf(cosI_));
    return f;
}
PLT_DI float fresnelR(const FresnelD& f) { return 0.5f * (f.rs * f.rs + f.rp * f.rp); }

PLT_NI void fresnel_conductor(float cosI, f2 eta, f2& rs, f2& rp) {
    if ((eta.x == 0.f && eta.y == 0.f) || cosI < 0.f) {
        rs = rp = f2{0.f, 0.f};
        return;
    }
    const f2 inv = cdiv(f2{1.f, 0.f}, eta);
    const f2 inv2 = cmul(inv, inv);
    const float s2 = 1.f - cosI * cosI;
    const f2 t = csqrt(f2{1.f - inv2.x * s2, -(inv2.y * s2)});
    const f2 et = cmul(eta, t);
    const f2 ei = f2{eta.x * cosI, eta.y * cosI};
    rs = cdiv(f2{cosI - et.x, -et.y}, f2{cosI + et.x, et.y});
    rp = cdiv(f2{ei.x - t.x, ei.y - t.y}, f2{ei.x + t.x, ei.y + t.y});
}

// ---- Fresnel Mueller matrices.  MuellerFresnel(fs, fp) (Mueller.slang:78-90) has the block form
//   [[a, b, 0, 0], [b, a, 0, 0], [0, 0, c, d], [0, 0, -d, c]]
// which is closed under products, sums and the inverse used by invOneMinusMuellerFresnel, so
// every Fresnel Mueller product of the PLT BSDFs is carried as four numbers (a, b, c, d).
// The reference forms c, d from the elementwise float2 product fs * cconj(fp): c = fs.x*fp.x,
// d = -fs.y*fp.y. ----
struct MM { float a, b, c, d; };
PLT_DI MM muellerFresnel(f2 fs, f2 fp) {
    const float Rp = cnorm2(fp), Rs = cnorm2(fs);
    return MM{(Rp + Rs) / 2.f, (Rp - Rs) / 2.f, fs.x * fp.x, fs.y * -fp.y};
}
PLT_DI MM muellerFresnelReal(float fs, float fp) {
    const float Rp = fp * fp, Rs = fs * fs;
    return MM{(Rp + Rs) / 2.f, (Rp - Rs) / 2.f, fs * fp, 0.f};
}
PLT_DI MM mmul(MM x, MM y) {
    return MM{x.a * y.a + x.b * y.b, x.a * y.b + x.b * y.a, x.c * y.c - x.d * y.d, x.c * y.d + x.d * y.c};
}
PLT_DI MM madd(MM x, MM y) { return MM{x.a + y.a, x.b + y.b, x.c + y.c, x.d + y.d}; }
PLT_DI f4 mapply(MM m, f4 s) { return f4{m.a * s.x + m.b * s.y, m.b * s.x + m.a * s.y, m.c * s.z + m.d * s.w, -m.d * s.z + m.c * s.w}; }
// invOneMinusMuellerFresnel (Mueller.slang:91-110), tryInvert threshold 4e-6 on each 2x2 block
PLT_DI bool invOneMinus(MM m, MM& out) {
    const float p00 = 1.f - m.a, p01 = 0.f - m.b;      // minor1 = I - [[a,b],[b,a]]
    const float q00 = 1.f - m.c, q01 = 0.f - m.d;      // minor2 = I - [[c,d],[-d,c]]
    const float q10 = 0.f - (-m.d);
    const float det1 = p00 * p00 - p01 * p01;
    const float det2 = q00 * q00 - q01 * q10;
    if (fabsf(det1) < 4e-6f || fabsf(det2) < 4e-6f) {
        out = MM{0.f, 0.f, 0.f, 0.f};
        return false;
    }
    const float i1 = 1.f / det1, i2 = 1.f / det2;
    out = MM{p00 * i1, -p01 * i1, q00 * i2, -q01 * i2};
    return true;
}
PLT_DI MM muellerRDielectric(float cosI, float eta) { const FresnelD f = fresnel_dielectric(cosI, eta); return muellerFresnelReal(f.rs, f.rp); }
PLT_DI MM muellerTDielectric(float cosI, float eta) { const FresnelD f = fresnel_dielectric(cosI, eta); return muellerFresnelReal(f.ts, f.tp); }

// fresnel_conductor evaluated in FP64 (the same expressions in double), rounded to FP32 at the end
PLT_NI void fresnel_conductor_f64(float cosIf, f2 etaf, f2& rs, f2& rp) {
    if ((etaf.x == 0.f && etaf.y == 0.f) || cosIf < 0.f) {
        rs = rp = f2{0.f, 0.f};
        return;
    }
    const double cosI = cosIf, ex = etaf.x, ey = etaf.y;
    const double den = ex * ex + ey * ey;
    const double ix = ex / den, iy = -ey / den;                    // 1 / eta
    const double i2x = ix * ix - iy * iy, i2y = 2.0 * ix * iy;      // (1 / eta)^2
    const double s2 = 1.0 - cosI * cosI;
    const double t2x = 1.0 - i2x * s2, t2y = -(i2y * s2);
    // csqrt as MathHelpers.slang writes it: (sqrt((r + x) / 2), sign(y) sqrt((r - x) / 2))
    const double m = sqrt(t2x * t2x + t2y * t2y);
    const double tx = sqrt(fmax(0.0, m + t2x) / 2.0);
    const double ty = (t2y > 0.0 ? 1.0 : (t2y < 0.0 ? -1.0 : 0.0)) * sqrt(fmax(0.0, m - t2x) / 2.0);
    const double etx = ex * tx - ey * ty, ety = ex * ty + ey * tx;  // eta t
    auto cdivd = [](double ax, double ay, double bx, double by, f2& out) {
        const double d = bx * bx + by * by;
        out = f2{(float)((ax * bx + ay * by) / d), (float)((ay * bx - ax * by) / d)};
    };
    cdivd(cosI - etx, -ety, cosI + etx, ety, rs);
    cdivd(ex * cosI - tx, ey * cosI - ty, ex * cosI + tx, ey * cosI + ty, rp);
}

// ---- complex-IOR conductor Fresnel: FP32 as the reference, or with PLT_OPTION_FP64_CONDUCTOR_GRAZING
// in FP64 below cos(theta_i) = kFp64GrazingCos (about 84.3 degrees) ----
constexpr float kFp64GrazingCos = 0.1f;
PLT_DI MM muellerRConductor(float cosI, f2 eta, f2& rs, f2& rp, uint32_t flags = 0u) {
    if ((flags & PLT_OPTION_FP64_CONDUCTOR_GRAZING) && cosI < kFp64GrazingCos) fresnel_conductor_f64(cosI, eta, rs, rp);
    else fresnel_conductor(cosI, eta, rs, rp);
    return muellerFresnel(rs, rp);
}

// ---- spectra ----
// rgbToSpectrum is precomputed per material on the host as an 11-bin table (the basis is
// piecewise constant over 11 bins of 380-720 nm); the device only evaluates the bin index.
PLT_DI int spectrumBin(float wl) { return (int)(clampf((wl - 380.0f) / (720.0f - 380.0f), 0.f, 1.f) * 10.f); }

}  // namespace pltdev
#include "plt_layout.h"
namespace pltdev {

PLT_NI float evalSpectrum(const DevProfile* __restrict__ profiles, uint32_t nprof, uint32_t id, float lambda) {
    if (id == kNoProfile || id >= nprof) return 0.f;
    const DevProfile& sp = profiles[id];
    const int bins = (int)sp.bins;
    const float x = (lambda - sp.minl) / (sp.maxl - sp.minl) * ((float)bins - 1.0f);
    const float i = floorf(x);
    const float w = x - i;
    if (lambda < sp.minl || lambda > sp.maxl) return 0.f;
    const int i0 = max(0, min(bins - 1, (int)i));
    const int i1 = max(0, min(bins - 1, (int)(i + 1.f)));
    return sp.intensity * lerpf(sp.pdf[i0], sp.pdf[i1], w);
}

// ---- sample generator: SplitMix64-seeded xoshiro128** ----
PLT_DI uint32_t interleave_32bit(uint32_t vx, uint32_t vy) {
    uint32_t x = vx & 0x0000ffffu, y = vy & 0x0000ffffu;
    x = (x | (x << 8)) & 0x00FF00FFu; x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u; x = (x | (x << 1)) & 0x55555555u;
    y = (y | (y << 8)) & 0x00FF00FFu; y = (y | (y << 4)) & 0x0F0F0F0Fu;
    y = (y | (y << 2)) & 0x33333333u; y = (y | (y << 1)) & 0x55555555u;
    return x | (y << 1);
}
PLT_DI uint64_t splitmix64_next(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// 16 rounds of the TEA block cipher on (v0, v1) with the fixed 128-bit key of
// Utils/Math/HashUtils.slang:59-71 (Wheeler & Needham's TEA); the first output word.
PLT_DI uint32_t teaSeed(uint32_t v0, uint32_t v1) {
    uint32_t sum = 0;
#pragma unroll 4
    for (int i = 0; i < 16; ++i) {
        sum += 0x9e3779b9u;
        v0 += ((v1 << 4) + 0xa341316cu) ^ (v1 + sum) ^ ((v1 >> 5) + 0xc8013ea4u);
        v1 += ((v0 << 4) + 0xad90777du) ^ (v0 + sum) ^ ((v0 >> 5) + 0x7e95761eu);
    }
    return v0;
}

// The render pass's two sample generators (sampleGenerator): UniformSampleGenerator (init) and,
// with tiny set, TinyUniformSampleGenerator (initTiny: Utils/Sampling/TinyUniformSampleGenerator
// .slang:50-70, a 32-bit LCG with the Numerical Recipes constants of Pseudorandom/LCG.slang, its
// state in s0).
struct SampleGen {
    uint32_t s0, s1, s2, s3;
    bool tiny = false;
    PLT_DI void init(uint32_t px, uint32_t py, uint32_t sampleNumber) {
        uint64_t st = ((uint64_t)sampleNumber << 32) | (uint64_t)interleave_32bit(px, py);
        const uint64_t a = splitmix64_next(st);
        const uint64_t b = splitmix64_next(st);
        s0 = (uint32_t)a; s1 = (uint32_t)(a >> 32); s2 = (uint32_t)b; s3 = (uint32_t)(b >> 32);
        tiny = false;
    }
    PLT_DI void initTiny(uint32_t px, uint32_t py, uint32_t sampleNumber) {
        s0 = teaSeed(interleave_32bit(px, py), sampleNumber);
        s1 = s2 = s3 = 0u;
        tiny = true;
    }
    PLT_DI void init(uint32_t px, uint32_t py, uint32_t sampleNumber, bool tinyGen) {
        if (tinyGen) initTiny(px, py, sampleNumber);
        else init(px, py, sampleNumber);
    }
    PLT_DI uint32_t next() {
        if (tiny) {
            s0 = 1664525u * s0 + 1013904223u;
            return s0;
        }
        const uint32_t result = __funnelshift_l(s0 * 5u, s0 * 5u, 7) * 9u;
        const uint32_t t = s1 << 9;
        s2 ^= s0; s3 ^= s1; s1 ^= s2; s0 ^= s3;
        s2 ^= t;
        s3 = __funnelshift_l(s3, s3, 11);
        return result;
    }
    PLT_DI float next1D() { return (float)(next() >> 8) * 0x1p-24f; }
};

// ---- BesselJ (MathHelpers.slang:851-885) ----
// n! for n < 13 (the reference's table); every partial product is exact in binary32
PLT_DI float factorialf(int n) {
    if (n < 0 || n >= 13) return 0.f;
    float f = 1.f;
    for (int i = 2; i <= n; ++i) f *= (float)i;
    return f;
}
PLT_NI float besselJ(int nu, float x) {
    const float t = (nu > 0 || ((-nu) % 2) == 0) ? 1.f : -1.f;
    nu = abs(nu);
    const float cutoff = (float)nu + 1.f;
    const float interp = cutoff / 10.f;
    const float laa = sqrtf(2.f / kPi / x) * cosf(x - (float)nu * kPi / 2.f - kPi / 4.f);
    if (nu >= 7 || fabsf(x) >= cutoff + interp) return laa * t;
    const float x2 = x * x, x4 = x2 * x2, x6 = x2 * x4, x8 = x4 * x4;
    const float s = 6.f * powf(x / 2.f, (float)nu);
    const float a = 1.f / (6.f * factorialf(nu));
    const float b = -x2 / (24.f * factorialf(nu + 1));
    const float c1 = 11.f * x8 - 864.f * (float)(6 + nu) *
                     (x6 - 12.f * (5.f + (float)nu) * (3.f * x4 + 32.f * (float)(4 + nu) * (-2.f * x2 + 27.f * (float)(3 + nu))));
    const float c = c1 / factorialf(6 + nu) * x4 * 5.652695401144601e-10f;
    const float saa = s * (a + b + c);
    return lerpf(saa, laa, fmaxf(0.f, fminf(1.f, .5f * (x - cutoff - interp) / interp))) * t;
}

}  // namespace pltdev
