// ORACLE -- test infrastructure only.  A CPU restatement of the PLTFalcor PLT BSDF hot path
// (Slang shaders, which cannot be compiled here: slangc is absent and the reference ships no CPU
// build), used only to check the CUDA kernels.  Templated on the real type R: float gives the
// FP32 reference, double the FP64 reference, CF the op-counting build.
//
// Parity pins: the restatement follows the reference line by line (citations per function, paths
// inside ssteinberg/PLTFalcor).  The reference has no PLT golden vectors or tests; physics
// known-answer tests in tests/ pin the pieces that have closed forms.
#pragma once

#include <type_traits>

#include "plt_math.hpp"
#include "../include/plt_gb300.h"

namespace plt_oracle {

constexpr int MAXH = (int)PLT_MAX_HWSS;

// ---------------------------------------------------------------------------------------------
// binary16 -> float (exact)
// ---------------------------------------------------------------------------------------------
inline float half_to_float(uint16_t h) {
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t exp = (h >> 10) & 0x1Fu;
    uint32_t man = h & 0x3FFu;
    uint32_t bits;
    if (exp == 0) {
        if (man == 0) {
            bits = sign;
        } else {
            // subnormal half: normalise
            int e = -1;
            do { ++e; man <<= 1; } while ((man & 0x400u) == 0);
            man &= 0x3FFu;
            bits = sign | ((uint32_t)(127 - 15 - e) << 23) | (man << 13);
        }
    } else if (exp == 31) {
        bits = sign | 0x7F800000u | (man << 13);
    } else {
        bits = sign | ((exp - 15 + 127) << 23) | (man << 13);
    }
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}

// ---------------------------------------------------------------------------------------------
// RNG: UniformSampleGenerator = SplitMix64 seeding of xoshiro128**.
// Utils/Sampling/UniformSampleGenerator.slang:51-66, Pseudorandom/SplitMix64.slang:54-78,
// Pseudorandom/Xoshiro.slang:52-113, SampleGeneratorInterface.slang:46-70, Math/BitTricks.slang:45-65
// ---------------------------------------------------------------------------------------------
inline uint32_t interleave_32bit(uint32_t vx, uint32_t vy) {
    uint32_t x = vx & 0x0000ffffu, y = vy & 0x0000ffffu;
    x = (x | (x << 8)) & 0x00FF00FFu; x = (x | (x << 4)) & 0x0F0F0F0Fu;
    x = (x | (x << 2)) & 0x33333333u; x = (x | (x << 1)) & 0x55555555u;
    y = (y | (y << 8)) & 0x00FF00FFu; y = (y | (y << 4)) & 0x0F0F0F0Fu;
    y = (y | (y << 2)) & 0x33333333u; y = (y | (y << 1)) & 0x55555555u;
    return x | (y << 1);
}
inline uint64_t splitmix64_next(uint64_t& state) {
    uint64_t z = (state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
inline uint32_t rotl32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }
// blockCipherTEA (Utils/Math/HashUtils.slang:59-71), 16 rounds; its first output word
inline uint32_t teaFirstWord(uint32_t v0, uint32_t v1) {
    const uint32_t k[4] = {0xa341316cu, 0xc8013ea4u, 0xad90777du, 0x7e95761eu};
    uint32_t sum = 0;
    for (int i = 0; i < 16; ++i) {
        sum += 0x9e3779b9u;
        v0 += ((v1 << 4) + k[0]) ^ (v1 + sum) ^ ((v1 >> 5) + k[1]);
        v1 += ((v0 << 4) + k[2]) ^ (v0 + sum) ^ ((v0 >> 5) + k[3]);
    }
    return v0;
}
// UniformSampleGenerator, or with tiny TinyUniformSampleGenerator
// (Utils/Sampling/TinyUniformSampleGenerator.slang:50-70: LCG, Pseudorandom/LCG.slang, seeded with
// blockCipherTEA(interleave_32bit(pixel), sampleNumber).x; its state in s[0]).
struct SampleGen {
    uint32_t s[4];
    bool tiny = false;
    SampleGen(uint32_t px, uint32_t py, uint32_t sampleNumber, bool tinyGen = false) {
        if (tinyGen) {
            tiny = true;
            s[0] = teaFirstWord(interleave_32bit(px, py), sampleNumber);
            s[1] = s[2] = s[3] = 0u;
            return;
        }
        uint64_t st = ((uint64_t)sampleNumber << 32) | (uint64_t)interleave_32bit(px, py);
        const uint64_t s0 = splitmix64_next(st);
        const uint64_t s1 = splitmix64_next(st);
        s[0] = (uint32_t)s0; s[1] = (uint32_t)(s0 >> 32); s[2] = (uint32_t)s1; s[3] = (uint32_t)(s1 >> 32);
    }
    uint32_t next() {
        if (tiny) {
            s[0] = 1664525u * s[0] + 1013904223u;
            return s[0];
        }
        const uint32_t result = rotl32(s[0] * 5u, 7) * 9u;
        const uint32_t t = s[1] << 9;
        s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl32(s[3], 11);
        return result;
    }
    float next1D() { return (float)(next() >> 8) * 0x1p-24f; }
};
template <class R> inline R next1D(SampleGen& sg) { return R((double)sg.next1D()); }
template <class R> inline V2<R> next2D(SampleGen& sg) { V2<R> u; u.x = next1D<R>(sg); u.y = next1D<R>(sg); return u; }
// Primary-sample warp of the surface models' direction samplers (the learned proposal of the
// path-tracing oracle): when set, the Gaussian and fractal surface samplers draw their pair as usual
// and then use this one instead.  Set and cleared around one sample call by the caller.
inline thread_local const float* g_directionWarp = nullptr;
template <class R> inline V2<R> nextDirection2D(SampleGen& sg) {
    V2<R> u = next2D<R>(sg);
    if (g_directionWarp) { u.x = R(g_directionWarp[0]); u.y = R(g_directionWarp[1]); }
    return u;
}

// ---------------------------------------------------------------------------------------------
// Spectra.  rgbToSpectrum: Utils/Color/SpectrumUtils.slang:106-198 (11-bin Smits-style basis over
// 380-720 nm; bin 10 is zero).  evalSpectrum: Scene/Scene.slang:251-294.
// ---------------------------------------------------------------------------------------------
struct SpectrumBasis {
    static constexpr float white[11] = {1.0000f, 1.0000f, 0.9999f, 0.9993f, 0.9992f, 0.9998f, 1.0000f, 1.0000f, 1.0000f, 1.0000f, 0.0f};
    static constexpr float cyan[11] = {0.9710f, 0.9426f, 1.0007f, 1.0007f, 1.0007f, 1.0007f, 0.1564f, 0.0000f, 0.0000f, 0.0000f, 0.0f};
    static constexpr float magenta[11] = {1.0000f, 1.0000f, 0.968f, 0.22295f, 0.0000f, 0.0458f, 0.8369f, 1.0000f, 1.0000f, 0.9959f, 0.0f};
    static constexpr float yellow[11] = {0.0001f, 0.0000f, 0.1088f, 0.6651f, 1.0000f, 1.0000f, 0.9996f, 0.9586f, 0.9685f, 0.9840f, 0.0f};
    static constexpr float red[11] = {0.1012f, 0.0515f, 0.0000f, 0.0000f, 0.0000f, 0.0000f, 0.8325f, 1.0149f, 1.0149f, 1.014f, 0.0f};
    static constexpr float green[11] = {0.0000f, 0.0000f, 0.0273f, 0.7937f, 1.0000f, 0.9418f, 0.1719f, 0.0000f, 0.0000f, 0.0025f, 0.0f};
    static constexpr float blue[11] = {1.0000f, 1.0000f, 0.8916f, 0.3323f, 0.0000f, 0.0000f, 0.0003f, 0.0369f, 0.0483f, 0.0496f, 0.0f};
};
constexpr float SPEC_MIN_WL = 380.0f, SPEC_MAX_WL = 720.0f, SPEC_MEAN_WL = 550.0f;

template <class R> inline int spectrum_bin(R wavelength) {
    const R t = o_clamp((wavelength - R(SPEC_MIN_WL)) / (R(SPEC_MAX_WL) - R(SPEC_MIN_WL)), R(0), R(1)) * R(10);
    return (int)t;
}
template <class R> inline R rgbToSpectrum(const R rgb[3], R wavelength) {
    using B = SpectrumBasis;
    const int b = spectrum_bin(wavelength);
    const R w = R(B::white[b]), c = R(B::cyan[b]), m = R(B::magenta[b]), y = R(B::yellow[b]);
    const R r = R(B::red[b]), g = R(B::green[b]), bl = R(B::blue[b]);
    R sd = R(0);
    if (rgb[0] <= rgb[1] && rgb[0] <= rgb[2]) {
        sd += w * rgb[0];
        if (rgb[1] <= rgb[2]) { sd += c * (rgb[1] - rgb[0]); sd += bl * (rgb[2] - rgb[1]); }
        else { sd += c * (rgb[2] - rgb[0]); sd += g * (rgb[1] - rgb[2]); }
    } else if (rgb[1] <= rgb[0] && rgb[1] <= rgb[2]) {
        sd += w * rgb[1];
        if (rgb[0] <= rgb[2]) { sd += m * (rgb[0] - rgb[1]); sd += bl * (rgb[2] - rgb[0]); }
        else { sd += m * (rgb[2] - rgb[1]); sd += r * (rgb[0] - rgb[2]); }
    } else {
        sd += w * rgb[2];
        if (rgb[0] <= rgb[1]) { sd += y * (rgb[0] - rgb[2]); sd += g * (rgb[1] - rgb[0]); }
        else { sd += y * (rgb[1] - rgb[2]); sd += r * (rgb[0] - rgb[1]); }
    }
    return sd;
}

struct SceneTables {
    const plt_spectral_profile* profiles = nullptr;
    uint32_t count = 0;
};
template <class R> inline R evalSpectrum(const SceneTables& sc, uint32_t id, R lambda) {
    if (id == PLT_NO_SPECTRAL_PROFILE || id >= sc.count) return R(0);
    const plt_spectral_profile& sp = sc.profiles[id];
    const int bins = (int)sp.bins;
    const R minl = R(sp.min_wavelength), maxl = R(sp.max_wavelength);
    const R x = (lambda - minl) / (maxl - minl) * (R((double)bins) - R(1));
    const R i = o_floor(x);
    const R w = x - i;
    if (lambda < minl || lambda > maxl) return R(0);
    const int ii = (int)i;
    const int i0 = std::max(0, std::min(bins - 1, ii));
    const int i1 = std::max(0, std::min(bins - 1, (int)(i + R(1))));
    return R(sp.intensity) * lerp(R(sp.pdf[i0]), R(sp.pdf[i1]), w);
}

// ---------------------------------------------------------------------------------------------
// Colour: CIE XYZ multi-lobe fit and the 5-nm D65 table of the shaders (SpectrumUtils.slang:43-82)
// ---------------------------------------------------------------------------------------------
inline float gaussLobe(float x, float lambda, float invSigma1, float invSigma2) {
    const float t = (x - lambda) * (x < lambda ? invSigma1 : invSigma2);
    return std::exp(-0.5f * t * t);
}
inline V3<float> wavelengthToXYZ(float l) {
    const float x = 0.362f * gaussLobe(l, 442.0f, 0.0624f, 0.0374f) + 1.056f * gaussLobe(l, 599.8f, 0.0264f, 0.0323f) -
                    0.065f * gaussLobe(l, 501.1f, 0.0490f, 0.0382f);
    const float y = 0.821f * gaussLobe(l, 568.8f, 0.0213f, 0.0247f) + 0.286f * gaussLobe(l, 530.9f, 0.0613f, 0.0322f);
    const float z = 1.217f * gaussLobe(l, 437.0f, 0.0845f, 0.0278f) + 0.681f * gaussLobe(l, 459.0f, 0.0385f, 0.0725f);
    return {x, y, z};
}
constexpr float kD65_5nm[69] = {49.9755f, 52.3118f, 54.6482f, 68.7015f, 82.7549f, 87.1204f, 91.486f, 92.4589f, 93.4318f, 90.057f,
                            86.6823f, 95.7736f, 104.865f, 110.936f, 117.008f, 117.41f, 117.812f, 116.336f, 114.861f, 115.392f,
                            115.923f, 112.367f, 108.811f, 109.082f, 109.354f, 108.578f, 107.802f, 106.296f, 104.79f, 106.239f,
                            107.689f, 106.047f, 104.405f, 104.225f, 104.046f, 102.023f, 100.f, 98.1671f, 96.3342f, 96.0611f,
                            95.788f, 92.2368f, 88.6856f, 89.3459f, 90.0062f, 89.8026f, 89.5991f, 88.6489f, 87.6987f, 85.4936f,
                            83.2886f, 83.4939f, 83.6992f, 81.863f, 80.0268f, 80.1207f, 80.2146f, 81.2462f, 82.2778f, 80.281f,
                            78.2842f, 74.0027f, 69.7213f, 70.6652f, 71.6091f, 72.979f, 74.349f, 67.9765f, 61.604f};
inline float wavelengthToD65(float l) {
    const float r = (l - SPEC_MIN_WL) * 0.2f;
    const int t = int(std::ceil(r) + .5f);
    const int b = int(std::floor(r) + .5f);
    const float w = r - float(b);
    return kD65_5nm[t] * w + kD65_5nm[b] * (1.0f - w);
}

// Profile colour for genSpectralProfile's sp.rgb = SpectrumUtils::toRGB_D65 (SceneBuilder.cpp:913,
// SpectrumUtils.h:78-151): trapezoid sum over the sampled spectrum of s * xyz * D65, XYZ -> Rec.709,
// / 10567.0762.  The colour-matching functions are the shaders' analytic fit and D65 the shaders'
// 5-nm table, zero outside 380-720 nm (the host's 1-nm CIE tables are not restated).
template <class SS> inline void profileRgb(float l0, float l1, size_t ns, SS ssEval, float rgb[3]) {
    const float delta = ns > 1 ? (l1 - l0) / (float(ns) - 1.0f) : 0.f;
    float X = 0.f, Y = 0.f, Z = 0.f;
    for (size_t q = 0; q < ns; ++q) {
        const float l = std::min(l0 + delta * float(q), l1);
        const float s = ssEval(l);
        const float d65 = (l >= SPEC_MIN_WL && l <= SPEC_MAX_WL) ? wavelengthToD65(l) : 0.f;
        const V3<float> xyz = wavelengthToXYZ(l);
        const float wq = s * delta * ((q == 0 || q == ns - 1) ? 0.5f : 1.0f);
        X += xyz.x * d65 * wq;
        Y += xyz.y * d65 * wq;
        Z += xyz.z * d65 * wq;
    }
    const float k = 1.0f / 10567.0762f;
    rgb[0] = (3.240969941904522f * X + -1.537383177570094f * Y + -0.4986107602930032f * Z) * k;
    rgb[1] = (-0.9692436362808803f * X + 1.875967501507721f * Y + 0.04155505740717569f * Z) * k;
    rgb[2] = (0.05563007969699373f * X + -0.2039769588889765f * Y + 1.056971514242878f * Z) * k;
}

// ---------------------------------------------------------------------------------------------
// Beam: PLTCoherence + PLTBeam, Rendering/PLT.slang:41-245
// ---------------------------------------------------------------------------------------------
template <class R> struct Beam {
    int H = 1;                       // hwss_comps (= hwss_samples in the batch API)
    R L[4][MAXH];                    // Stokes planes L, L1, L2, L3
    R wl[MAXH];
    R spdf[MAXH];
    R D[3];                          // diffusivity (D00, D01, D11)
    R r_m;                           // distance from source (m)
    V3<R> posW, r, t;
    bool distant = false;

    V4<R> getSP(int j) const { return {L[0][j], L[1][j], L[2][j], L[3][j]}; }
    void setSP(int j, V4<R> s) { L[0][j] = s.x; L[1][j] = s.y; L[2][j] = s.z; L[3][j] = s.w; }
    void setZero() { for (int c = 0; c < 4; ++c) for (int j = 0; j < H; ++j) L[c][j] = R(0); }
    void scale(const R* s) { for (int c = 0; c < 4; ++c) for (int j = 0; j < H; ++j) L[c][j] *= s[j]; }

    R rmm() const { return r_m * R(1e+3); }
    M2<R> diffMat() const { return m2(D[0], D[1], D[1], D[2]); }
    // toInvCoherenceMat(k), PLT.slang:57-60
    M2<R> invTheta(R k) const {
        const R recp_lambda = k / R(K_2PI);
        return sqr(recp_lambda / rmm()) * diffMat();
    }
    // toInvCoherenceMat(), PLT.slang:61-63
    M2<R> invTheta() const { return sqr(R(1) / rmm()) * diffMat(); }
    R det(R k) const { return R(1) / determinant(invTheta(k)); }

    // Q(), PLT.slang:146-150
    M2<R> Q() const {
        const V3<R> b = cross(t, r);
        return transpose(m2(t.x, t.y, b.x, b.y));
    }
    // mutualCoherence (scalar k), PLT.slang:159-163
    R mutualCoherence(R k, V3<R> v) const {
        const M2<R> iT = invTheta(k);
        const V2<R> vx = {v.x, v.y};
        const R x = dot(vx, mul(iT, vx));
        return o_exp(R(-0.5) * x);
    }
    // mutualCoherence (hwss k), PLT.slang:164-169
    void mutualCoherenceH(const R* k, V3<R> v, R* out) const {
        const M2<R> iT = invTheta();
        const V2<R> vx = {v.x, v.y};
        const R d = dot(vx, mul(iT, vx));
        for (int j = 0; j < H; ++j) {
            const R recp = k[j] / R(K_2PI);
            out[j] = o_exp(R(-0.5) * (sqr(recp) * d));
        }
    }
    // mutualCoherenceAngular, PLT.slang:172-177
    R mutualCoherenceAngular(V3<R> d1, V3<R> d2) const {
        const R s4 = o_sqrt(R(K_4PI));
        const V2<R> v = {R(1) / o_max(s4 * o_abs(d1.x - d2.x), R(K_FLT_EPSILON)),
                         R(1) / o_max(s4 * o_abs(d1.y - d2.y), R(K_FLT_EPSILON))};
        const M2<R> iT = invTheta() * sqr(rmm());
        const R x = R(1) / dot(v, mul(iT, v));
        return o_exp(R(-0.5) * x);
    }
    R coherenceArea(R k) const { return R(K_PI) * o_sqrt(det(k)); }

    // transformCoherence / PLTCoherence.transform, PLT.slang:73-77,200-202
    void transformCoherence(M2<R> U) {
        const M2<R> Dm = diffMat();
        const M2<R> nD = mul(transpose(U), mul(Dm, U));
        D[0] = nD.m[0][0]; D[1] = nD.m[0][1]; D[2] = nD.m[1][1];
    }
    // rotateFrame, PLT.slang:203-216 with MuellerT, Mueller.slang:34-53
    void rotateFrame(V3<R> newt, V3<R> newr) {
        R theta = o_atan2(dot(r, cross(t, newt)), dot(t, newt));
        theta = o_isfinite(theta) ? theta : R(0);
        const R sint = o_sin(theta), cost = o_cos(theta);
        const R rx = R(2) * sint * cost;
        const R ry = R(1) - R(2) * sqr(sint);
        for (int j = 0; j < H; ++j) {
            const V4<R> s = getSP(j);
            // T = [[1,0,0,0],[0,rx,-ry,0],[0,ry,rx,0],[0,0,0,1]] (MuellerT, Mueller.slang:46-50)
            const V4<R> n = {s.x, rx * s.y + (-ry) * s.z, ry * s.y + rx * s.z, s.w};
            setSP(j, n);
        }
        transformCoherence(m2(cost, -sint, sint, cost));
        r = newr;
        t = newt;
    }
    // constructLocalFrame, PLT.slang:218-223
    void constructLocalFrame(V3<R> newwo) {
        V3<R> newt = cross(V3<R>{R(0), R(0), R(1)}, newwo);
        const R l2 = dot(newt, newt);
        newt = l2 > R(1e-8) ? newt / o_sqrt(l2) : perp_stark(newwo);
        rotateFrame(newt, newwo);
    }
    V3<R> toLocal(V3<R> v) const { return {dot(v, t), dot(v, cross(t, r)), dot(v, r)}; }
};

// canonical beam tangent of direction r (the frame constructLocalFrame builds)
template <class R> inline V3<R> canonical_tangent(V3<R> r) {
    V3<R> t = cross(V3<R>{R(0), R(0), R(1)}, r);
    const R l2 = dot(t, t);
    return l2 > R(1e-8) ? t / o_sqrt(l2) : perp_stark(r);
}

// ---------------------------------------------------------------------------------------------
// Fresnel, Rendering/Materials/Fresnel.slang:30-90
// ---------------------------------------------------------------------------------------------
template <class R> inline void fresnel_dielectric(R cosThetaI_, R eta, R& rs, R& rp, R& ts, R& tp, R& cosThetaT) {
    if (eta == R(1)) {
        cosThetaT = -cosThetaI_;
        rs = rp = R(0);
        ts = tp = R(1);
        return;
    }
    eta = (cosThetaI_ > R(0)) ? eta : R(1) / eta;
    const R cosThetaI = o_abs(cosThetaI_);
    const R cosThetaTSqr = R(1) - (R(1) - sqr(cosThetaI)) / sqr(eta);
    cosThetaT = o_sqrt(o_max(R(0), cosThetaTSqr));
    rs = (cosThetaI - eta * cosThetaT) / (cosThetaI + eta * cosThetaT);
    rp = (eta * cosThetaI - cosThetaT) / (eta * cosThetaI + cosThetaT);
    const R imp = o_sqrt(eta * cosThetaT / cosThetaI);
    ts = imp * (rs + R(1));
    tp = imp * (rp + R(1)) / eta;
    cosThetaT = cosThetaT * (-o_sign(cosThetaI_));
}
template <class R> inline R evalFresnelDielectric(R eta, R cosThetaI, R& cosThetaT) {
    R rs, rp, ts, tp;
    fresnel_dielectric(cosThetaI, eta, rs, rp, ts, tp, cosThetaT);
    return R(0.5) * (sqr(rs) + sqr(rp));
}
template <class R> inline R evalFresnelDielectric(R eta, R cosThetaI) { R c; return evalFresnelDielectric(eta, cosThetaI, c); }

// The FP32 oracle's twin of PLT_OPTION_FP64_CONDUCTOR_GRAZING: set per thread around a query.
inline thread_local bool g_fp64ConductorGrazing = false;
constexpr float kFp64GrazingCos = 0.1f;
template <class R> inline void fresnel_conductor(R cosThetaI, V2<R> eta, V2<R>& rs, V2<R>& rp);
template <class R> inline void fresnel_conductor(R cosThetaI, V2<R> eta, V2<R>& rs, V2<R>& rp) {
    if constexpr (std::is_same_v<R, float>) {
        if (g_fp64ConductorGrazing && cosThetaI < kFp64GrazingCos) {
            V2<double> a, b;
            fresnel_conductor<double>((double)cosThetaI, V2<double>{(double)eta.x, (double)eta.y}, a, b);
            rs = V2<float>{(float)a.x, (float)a.y};
            rp = V2<float>{(float)b.x, (float)b.y};
            return;
        }
    }
    if ((eta.x == R(0) && eta.y == R(0)) || cosThetaI < R(0)) {
        rs = rp = c_t(R(0), R(0));
        return;
    }
    const V2<R> inv = cdiv(c_t(R(1)), eta);
    const V2<R> t2 = c_t(R(1)) - csqr(inv) * (R(1) - sqr(cosThetaI));
    const V2<R> t = csqrt(t2);
    const V2<R> i = c_t(cosThetaI);
    rs = cdiv(i - cmul(eta, t), i + cmul(eta, t));
    rp = cdiv(cmul(eta, i) - t, cmul(eta, i) + t);
}
template <class R> inline R evalFresnelConductor(V2<R> eta, R cosThetaI) {
    V2<R> rs, rp;
    fresnel_conductor(cosThetaI, eta, rs, rp);
    return R(0.5) * (cnorm2(rs) + cnorm2(rp));
}

// ---------------------------------------------------------------------------------------------
// Mueller matrices, Rendering/Materials/PLT/Mueller.slang:78-144.
// Note: MuellerFresnel forms m22/m23 from the ELEMENTWISE float2 product fs*cconj(fp)
// (Mueller.slang:82-83); that is what the reference computes and what parity follows.
// ---------------------------------------------------------------------------------------------
template <class R> inline M4<R> MuellerFresnel(V2<R> fs, V2<R> fp) {
    const R Rp = cnorm2(fp), Rs = cnorm2(fs);
    const R m00 = (Rp + Rs) / R(2), m01 = (Rp - Rs) / R(2);
    const V2<R> cf = cconj(fp);
    const R m22 = fs.x * cf.x;
    const R m23 = fs.y * cf.y;
    M4<R> M = zero4<R>();
    M.m[0][0] = m00; M.m[0][1] = m01; M.m[1][0] = m01; M.m[1][1] = m00;
    M.m[2][2] = m22; M.m[2][3] = m23; M.m[3][2] = -m23; M.m[3][3] = m22;
    return M;
}
template <class R> inline M4<R> invOneMinusMuellerFresnel(V2<R> fs, V2<R> fp) {
    const R Rp = cnorm2(fp), Rs = cnorm2(fs);
    const R m00 = (Rp + Rs) / R(2), m01 = (Rp - Rs) / R(2);
    const V2<R> cf = cconj(fp);
    const R m22 = fs.x * cf.x;
    const R m23 = fs.y * cf.y;
    const M2<R> minor1 = m2(R(1), R(0), R(0), R(1)) - m2(m00, m01, m01, m00);
    const M2<R> minor2 = m2(R(1), R(0), R(0), R(1)) - m2(m22, m23, -m23, m22);
    M2<R> im1, im2;
    if (!tryInvert(minor1, im1) || !tryInvert(minor2, im2)) return zero4<R>();
    M4<R> M = zero4<R>();
    M.m[0][0] = im1.m[0][0]; M.m[0][1] = im1.m[0][1]; M.m[1][0] = im1.m[0][1]; M.m[1][1] = im1.m[0][0];
    M.m[2][2] = im2.m[0][0]; M.m[2][3] = im2.m[0][1]; M.m[3][2] = im2.m[1][0]; M.m[3][3] = im2.m[0][0];
    return M;
}
template <class R> inline M4<R> MuellerFresnelRConductor(R cosThetaI, V2<R> eta, V2<R>& rs, V2<R>& rp) {
    fresnel_conductor(cosThetaI, eta, rs, rp);
    return MuellerFresnel(rs, rp);
}
template <class R> inline M4<R> MuellerFresnelRConductor(R cosThetaI, V2<R> eta) { V2<R> a, b; return MuellerFresnelRConductor(cosThetaI, eta, a, b); }
template <class R> inline M4<R> MuellerFresnelRDielectric(R cosThetaI, R eta) {
    R rs, rp, ts, tp, c;
    fresnel_dielectric(cosThetaI, eta, rs, rp, ts, tp, c);
    return MuellerFresnel(c_t(rs, R(0)), c_t(rp, R(0)));
}
template <class R> inline M4<R> invOneMinusMuellerFresnelRDielectric(R cosThetaI, R eta) {
    R rs, rp, ts, tp, c;
    fresnel_dielectric(cosThetaI, eta, rs, rp, ts, tp, c);
    return invOneMinusMuellerFresnel(c_t(rs, R(0)), c_t(rp, R(0)));
}
template <class R> inline M4<R> MuellerFresnelTDielectric(R cosThetaI, R eta) {
    R rs, rp, ts, tp, c;
    fresnel_dielectric(cosThetaI, eta, rs, rp, ts, tp, c);
    return MuellerFresnel(c_t(ts, R(0)), c_t(tp, R(0)));
}
template <class R> inline M4<R> MuellerFresnelDielectric(R cosThetaI, R eta, bool reflection) {
    return reflection ? MuellerFresnelRDielectric(cosThetaI, eta) : MuellerFresnelTDielectric(cosThetaI, eta);
}
// MuellerPolarizer, Mueller.slang:57-73
template <class R> inline M4<R> MuellerPolarizer(R theta) {
    const R s = o_sin(theta), c = o_cos(theta);
    M4<R> P = zero4<R>();
    P.m[0][0] = R(1);
    P.m[0][1] = P.m[1][0] = c;
    P.m[0][2] = P.m[2][0] = s;
    P.m[1][2] = P.m[2][1] = c * s;
    P.m[1][1] = c * c;
    P.m[2][2] = s * s;
    P.m[3][3] = R(0);
    return R(0.5) * P;
}

// ---------------------------------------------------------------------------------------------
// Interference, Rendering/Materials/PLT/Interference.slang:36-57
// ---------------------------------------------------------------------------------------------
template <class R> inline R phaseShift(R eta, R dist, R k, V2<R> r) { return o_sin(dist * k * eta + carg(r)); }
template <class R> inline R phaseShiftH(R eta, R dist, R k) { return o_sin(dist * k * eta); }
template <class R> inline V4<R> interfere(V4<R> SP1, V4<R> SP2, R phasor_s, R phasor_p, R coh) {
    const R S1 = (SP1.x + SP1.y) / R(2), P1 = (SP1.x - SP1.y) / R(2);
    const R S2 = (SP2.x + SP2.y) / R(2), P2 = (SP2.x - SP2.y) / R(2);
    const R S = S1 + S2 + R(2) * o_sqrt(o_max(R(0), S1 * S2)) * phasor_s * coh;
    const R P = P1 + P2 + R(2) * o_sqrt(o_max(R(0), P1 * P2)) * phasor_p * coh;
    const R n = SP1.x + SP2.x > R(1e-6) ? (S + P) / (SP1.x + SP2.x) : R(0);
    return {S + P, S - P, (SP1.z + SP2.z) * n, (SP1.w + SP2.w) * n};
}

// ---------------------------------------------------------------------------------------------
// GaussianSurface, Rendering/Materials/PLT/GaussianSurface.slang:37-110
// ---------------------------------------------------------------------------------------------
template <class R> struct GaussianSurface {
    R sigma2, q;
    static R roughnessToSigma2(R r) { return o_pow(o_clamp(R(1) - R(0.5) * r, R(0), R(1)), R(28)) * R(2500); }
    explicit GaussianSurface(R psd) {
        const R s2 = roughnessToSigma2(psd);
        const R s2max = roughnessToSigma2(R(0.1));
        const R s2r0 = roughnessToSigma2(R(0));
        q = lerp(R(0), R(1), (s2r0 - s2) / (s2r0 - s2max));
        sigma2 = o_min(s2max, s2);
    }
    bool isDeltaOnly() const { return q == R(0); }
    R alpha(V3<R> wi, V3<R> wo, R k) const {
        const R a = sqr((o_abs(wi.z) + o_abs(wo.z)) * q * k);
        return isDeltaOnly() ? R(1) : o_exp(-a);
    }
    R alpha(V3<R> wi, R k) const { return alpha(wi, wi, k); }
    V3<R> sample(V3<R> wi, SampleGen& sg, R k, R& pdf) const {
        const R w = R(1) / sigma2;
        const R s2 = w / sqr(k);
        const V2<R> mean = {-wi.x, -wi.y};
        const V2<R> wo = sample_boxmueller_truncated(nextDirection2D<R>(sg), mean, s2, pdf);
        const R z = o_sqrt(o_max(R(0), R(1) - dot(wo, wo)));
        return {wo.x, wo.y, o_sign(wi.z) * z};
    }
    R pdf(V3<R> wi, V3<R> wo, R k) const {
        const R w = R(1) / sigma2;
        const R s2 = w / sqr(k);
        return boxmueller_truncated_pdf(V2<R>{wo.x, wo.y}, V2<R>{-wi.x, -wi.y}, s2);
    }
    R eval(R k, M2<R> invTheta, M2<R> Q, V3<R> h) const {
        invTheta = mul(Q, mul(invTheta, transpose(Q)));
        const M2<R> S = ident2<R>() / sigma2 + invTheta;
        const R d = determinant(S);
        const M2<R> invS = m2(S.m[1][1], -S.m[0][1], -S.m[1][0], S.m[0][0]) / d;
        const V2<R> hx = {h.x, h.y};
        return o_exp(R(-0.5) * sqr(k) * dot(hx, mul(invS, hx))) * (sqr(k) * R(K_1_2PI) / o_sqrt(d));
    }
};

// ---------------------------------------------------------------------------------------------
// FractalSurface, Rendering/Materials/PLT/FractalSurface.slang:38-135
// ---------------------------------------------------------------------------------------------
template <class R> inline R meank() { return R(K_2PI) / (R(SPEC_MEAN_WL) * R(1e-3)); }
template <class R> struct FractalSurface {
    R T, gamma;
    static R roughnessToT(R alpha) {
        const R alpha2 = sqr(o_clamp(alpha, R(0), R(0.75)));
        return o_min(R(5000), (R(1) - alpha2) / (R(4) * sqr(meank<R>()) * alpha2));
    }
    static R TToRoughness(R T) { return R(1) / o_sqrt(R(1) + R(4) * sqr(meank<R>()) * T); }
    FractalSurface(R psd, R g = R(3)) {
        gamma = o_max(R(1.1), g);
        T = roughnessToT(psd);
    }
    R roughness() const { return TToRoughness(T); }
    R q() const { return roughness() * R(1); }
    bool isDeltaOnly() const { return q() == R(0); }
    R alpha(V3<R> wi, V3<R> wo, R k) const { return o_exp(-sqr((o_abs(wi.z) + o_abs(wo.z)) * q() * k)); }
    R alpha(V3<R> wi, R k) const { return alpha(wi, wi, k); }
    R pGF(V2<R> z) const {
        const R f = R(1) / o_pow(R(1) + T * dot(z, z), (gamma + R(1)) / R(2));
        return R(K_1_2PI) * (gamma - R(1)) * T * f;
    }
    V3<R> sample(V3<R> wi, SampleGen& sg, R k, R& pdf) const {
        const R s = o_sqrt(o_max(R(0), R(1) - sqr(wi.z)));
        const R phi_i = s > R(0) ? o_atan2(wi.y, wi.x) : R(0);
        const R sqrtT = o_sqrt(T);
        const V2<R> u1 = nextDirection2D<R>(sg);
        const V2<R> u2 = next2D<R>(sg);
        (void)u2;
        const R M = R(1) - o_pow(R(1) + sqr(k) * T * sqr(R(1) + s), -(gamma - R(1)) / R(2));
        const R f = o_sqrt(o_pow(R(1) - M * u1.x, R(-2) / (gamma - R(1))) - R(1)) / sqrtT;
        const R phi_max = (f == R(0) || s == R(0))
                              ? R(K_PI)
                              : o_acos(o_clamp((sqr(f / k) + sqr(s) - R(1)) / (R(2) * (f / k) * s), R(-1), R(1)));
        const R phi_f = phi_i + (R(2) * u1.y - R(1)) * phi_max;
        const V2<R> vf = {f * o_cos(phi_f), f * o_sin(phi_f)};
        const V2<R> wo = vf / k - V2<R>{wi.x, wi.y};
        const R z = o_sqrt(o_max(R(0), R(1) - dot(wo, wo)));
        pdf = R(K_PI) / phi_max * z * pGF(vf);
        return {wo.x, wo.y, o_sign(wi.z) * z};
    }
    R pdf(V3<R> wi, V3<R> wo, R k) const { return pGF(V2<R>{(wi.x + wo.x) * k, (wi.y + wo.y) * k}); }
    R eval(R k, V3<R> h) const { return pGF(V2<R>{h.x * k, h.y * k}); }
};

// ---------------------------------------------------------------------------------------------
// DiffractionGrating, Rendering/Materials/PLT/DiffractionGrating.slang:41-195 (.slangh:33-42)
// ---------------------------------------------------------------------------------------------
template <class R> struct DiffractionGrating {
    V2<R> gratingX, invPitch;
    R q;
    unsigned lobeCount, type;
    R intensityMultiplier;
    bool is1D() const { return invPitch.y == R(0); }
    R alpha(V3<R> wi, R k) const { return o_exp(-sqr(wi.z * q * k)); }
    R lobeIntensity(int lx, int ly, V3<R> wi, R lambda) const {
        const unsigned gt = type & 0xFu;
        const R a = R(K_4PI) * q / (lambda * o_abs(wi.z));
        R ix, iy;
        if (gt == 0u) {
            iy = ix = lx == 0 ? R(1) : BesselJ(lx, a);
            if (!is1D()) iy = ly == 0 ? R(1) : BesselJ(ly, a);
        } else if (gt == 1u) {
            iy = ix = lx == 0 ? R(1) : o_sin(a / R(2)) * sinc(R(K_PI) * R((double)lx) / R(2));
            if (!is1D()) iy = ly == 0 ? R(1) : o_sin(a / R(2)) * sinc(R(K_PI) * R((double)ly) / R(2));
        } else {
            iy = ix = lx == 0 ? R(1) : R(1) / o_sqrt(R((double)std::abs(lx)));
            if (!is1D()) iy = ly == 0 ? R(1) : R(1) / o_sqrt(R((double)std::abs(ly)));
        }
        return intensityMultiplier * ix * iy;
    }
    // closestLobeHint, DiffractionGrating.slang:92-107: the diffraction order whose direction is
    // closest to -woHint (manifold walks pass the direction towards the next path vertex)
    void closestLobeHint(V3<R> wi, V3<R> woHint, R alpha, R lambda, int& lx, int& ly) const {
        lx = ly = 0;
        if (alpha == R(1)) return;
        const R li2x = sqr(wi.x) + sqr(wi.z), li2y = sqr(wi.y) + sqr(wi.z);
        const R lo2x = sqr(woHint.x) + sqr(woHint.z), lo2y = sqr(woHint.y) + sqr(woHint.z);
        const R six = li2x > R(K_FLT_EPSILON) ? wi.x / o_sqrt(li2x) : R(0);
        const R siy = li2y > R(K_FLT_EPSILON) ? wi.y / o_sqrt(li2y) : R(0);
        const R sox = lo2x > R(K_FLT_EPSILON) ? -woHint.x / o_sqrt(lo2x) : R(0);
        const R soy = lo2y > R(K_FLT_EPSILON) ? -woHint.y / o_sqrt(lo2y) : R(0);
        auto toLobe = [&](R l) {
            const R v = l + o_sign(l) * R(0.5);
            const double dv = (double)o_fval(v);
            int li = std::isfinite(dv) ? (int)std::max(-1e9, std::min(1e9, dv)) : 0;
            return std::max(-(int)lobeCount, std::min((int)lobeCount, li));
        };
        const R l0 = (six - sox) / (invPitch.x * lambda);
        lx = toLobe(l0);
        if (alpha == R(0) && lx == 0) lx = (int)o_fval(o_sign(l0));
        if (!is1D()) {
            const R l1 = (siy - soy) / (invPitch.y * lambda);
            ly = toLobe(l1);
            if (alpha == R(0) && ly == 0) ly = (int)o_fval(o_sign(l1));
        }
    }
    // sampleLobe, :109-140
    void sampleLobe(V3<R> wi, int& lx, int& ly, V2<R>& pdf, R lambda, SampleGen& sg) const {
        R intensity[16];
        R total = R(0);
        for (int l = 0; l < (int)lobeCount; ++l) {
            const R li = lobeIntensity(l + 1, 0, wi, lambda);
            total += li;
            intensity[l] = li;
        }
        const V2<R> u = next2D<R>(sg);
        const V2<R> rnd = {(u.x - R(0.5)) * R(2), (u.y - R(0.5)) * R(2)};
        R cdf = R(0);
        lx = ly = 0;
        pdf = {R(0), R(0)};
        for (int l = 0; l < (int)lobeCount; ++l) {
            const R p = intensity[l] / total;
            cdf += p;
            const bool sx = o_abs(rnd.x) < cdf && lx == 0;
            const bool sy = o_abs(rnd.y) < cdf && ly == 0;
            if (sx) { pdf.x = p; lx = l + 1; }
            if (sy) { pdf.y = p; ly = l + 1; }
        }
        pdf = pdf / R(2);
        if (rnd.x < R(0)) lx = -lx;
        if (rnd.y < R(0)) ly = -ly;
        if (is1D()) { ly = 0; pdf.y = R(1); }
    }
    // diffract, :142-156
    V3<R> diffract(V3<R> wi, int lx, int ly, R lambda) const {
        const V2<R> p = {o_sqrt(sqr(wi.x) + sqr(wi.z)), o_sqrt(sqr(wi.y) + sqr(wi.z))};
        const V2<R> sini = {p.x > R(K_FLT_EPSILON) ? wi.x / p.x : R(0), p.y > R(K_FLT_EPSILON) ? wi.y / p.y : R(0)};
        const V2<R> sino = {lambda * R((double)lx) * invPitch.x - sini.x, lambda * R((double)ly) * invPitch.y - sini.y};
        const R a = sino.x, b = sino.y;
        const R m = (sqr(a) - R(1)) / (sqr(a * b) - R(1));
        const R qq = R(1) - sqr(b) * m;
        if (o_abs(sino.x) <= R(1) && o_abs(sino.y) <= R(1))
            return {a * o_sqrt(o_max(R(0), qq)), b * o_sqrt(m), o_sqrt(o_max(R(0), R(1) - sqr(a) * qq - sqr(b) * m))};
        return {R(0), R(0), R(0)};
    }
};

// grating lobe code in LobeType::MaterialSpecific bits, PLTDiffractionGrated*BSDF.slang:54-66
inline void encodeGratingLobe(int lx, int ly, uint32_t& bsdfLobe) {
    const int sx = lx < 0 ? 0 : 1, sy = ly < 0 ? 0 : 1;
    lx = std::min(std::abs(lx), 7);
    ly = std::min(std::abs(ly), 7);
    bsdfLobe &= ~(uint32_t)PLT_LOBE_MATERIAL_SPECIFIC;
    bsdfLobe += (uint32_t)(((ly << 3) + lx + (sy << 7) + (sx << 6)) << 8);
}
inline void decodeGratingLobe(uint32_t bsdfLobe, int& lx, int& ly) {
    const int x = (int)bsdfLobe >> 8;
    lx = x & 0x7;
    ly = (x >> 3) & 0x7;
    lx *= 2 * ((x >> 6) & 0x1) - 1;
    ly *= 2 * ((x >> 7) & 0x1) - 1;
}

// ---------------------------------------------------------------------------------------------
// Birefringence, Rendering/Materials/PLT/Birefringence.slang:33-197
// ---------------------------------------------------------------------------------------------
template <class R> struct Biref {
    static R qo(R eo, R K) { const R k = R(1); return o_sqrt(sqr(eo) * sqr(k) - sqr(K)); }
    static V2<R> qe(R eo, R ee, V3<R> A, R K) {
        const R e = sqr(ee) - sqr(eo);
        const R k = R(1);
        const R a = A.x, b = A.y, c = A.z;
        const R G = sqr(b) * e + sqr(eo);
        const R root = o_sqrt(o_max(R(0), sqr(K) * (sqr(a) * e - sqr(ee)) + sqr(k) * sqr(ee) * G));
        const R qep = (eo * root + c * b * K * e) / G;
        const R qem = (-eo * root + c * b * K * e) / G;
        return {qep, qem};
    }
    static V3<R> E_e(R eo, R ee, V3<R> A, R K, R q) {
        const R k = R(1);
        const R a = A.x, b = A.y, c = A.z;
        const V3<R> E = {a * sqr(k) * sqr(eo), K * c * q + b * (sqr(eo) * sqr(k) - sqr(q)), K * b * q + c * (sqr(eo) * sqr(k) - sqr(K))};
        return normalize(E);
    }
    static V3<R> E_ep(R eo, R ee, V3<R> A, R K) { return E_e(eo, ee, A, K, qe(eo, ee, A, K).x); }
    static V3<R> E_em(R eo, R ee, V3<R> A, R K) { return E_e(eo, ee, A, K, qe(eo, ee, A, K).y); }
    static V3<R> E_o(V3<R> A, R K, R q) {
        const R a = A.x, b = A.y, c = A.z;
        return normalize(V3<R>{-b * K - c * q, a * K, a * q});
    }
    static V3<R> E_op(R eo, V3<R> A, R K) { return E_o(A, K, qo(eo, K)); }
    static V3<R> E_om(R eo, V3<R> A, R K) { return E_o(A, K, -qo(eo, K)); }
    static V3<R> Poynting(R q, V3<R> E, R K) {
        return normalize(V3<R>{E.x * (K * E.z - q * E.y), K * E.z * E.y + q * (sqr(E.x) + sqr(E.z)),
                               -q * E.z * E.y - K * (sqr(E.x) + sqr(E.y))});
    }
    static void fresnel_iso_aniso(R cos_theta, R sin_theta, R ei, R eo, R ee, V3<R> A, R& rss, R& rsp, R& tso, R& tse,
                                  R& rps, R& rpp, R& tpo, R& tpe) {
        const R k = R(1);
        const R K = k * ei * sin_theta;
        const R qi = -qo(ei, K);
        const V3<R> E2om = E_om(eo, A, K);
        const V3<R> E2em = E_em(eo, ee, A, K);
        const R q2om = -qo(eo, K);
        const R q2em = qe(eo, ee, A, K).y;
        const R A_1 = -E2em.x * E2om.y * K * cos_theta;
        const R A_2 = -E2em.y * E2om.x * K * cos_theta;
        const R C_1 = qi * cos_theta - K * sin_theta;
        const R C_2 = E2em.x * E2om.z * (C_1 + q2om * cos_theta) - A_1;
        const R C_3 = E2em.z * E2om.x * (C_1 + q2em * cos_theta) - A_2;
        const R Ns = C_2 * (qi + q2em) - C_3 * (qi + q2om);
        rps = (R(2) * E2em.x * E2om.x * cos_theta * C_1 * (q2om - q2em)) / Ns;
        rpp = (-E2em.x * E2om.z * (C_1 - q2om * cos_theta) * (qi + q2em) + E2em.z * E2om.x * (C_1 - q2em * cos_theta) * (qi + q2om) -
               A_1 * (q2em + qi) + A_2 * (q2om + qi)) / Ns;
        tpo = -(R(2) * E2em.x * cos_theta * (q2em + qi) * C_1) / Ns;
        tpe = (R(2) * E2om.x * cos_theta * (q2om + qi) * C_1) / Ns;
        rss = (C_2 * (qi - q2em) + C_3 * (q2om - qi)) / Ns;
        rsp = (R(2) * qi * (E2em.z * E2om.y * K - E2em.y * E2om.z * K + E2em.z * E2om.z * (q2om - q2em))) / Ns;
        tso = -(R(2) * qi * (E2em.y * K * cos_theta + E2em.z * C_1 + E2em.z * q2em * cos_theta)) / Ns;
        tse = (R(2) * qi * (E2om.y * K * cos_theta + E2om.z * C_1 + E2om.z * q2om * cos_theta)) / Ns;
    }
    static void fresnel_aniso_iso(R cos_phi, R sin_phi, R ei, R eo, R ee, V3<R> A, R& roo, R& roe, R& tos, R& top, R& reo,
                                  R& ree, R& tes, R& tep) {
        const R eo2 = ei;
        const R k = R(1);
        const R K = k * ei * sin_phi;
        const R q2om = -qo(eo2, K);
        const R qop = qo(eo, K);
        const V2<R> q_e = qe(eo, ee, A, K);
        const R qep = q_e.x, qem = q_e.y;
        const V3<R> Eop = E_op(eo, A, K);
        const V3<R> Eep = E_ep(eo, ee, A, K);
        const V3<R> Eom = E_om(eo, A, K);
        const V3<R> Eem = E_em(eo, ee, A, K);
        const R B_1 = -Eep.x * K * cos_phi * (q2om - qep);
        const R B_2 = -Eom.x * K * cos_phi * (q2om + qop);
        const R B_3 = -Eop.x * K * cos_phi * (qop - q2om);
        const R D_1 = K * sin_phi - q2om * cos_phi;
        const R D_2 = Eep.z * (D_1 + qep * cos_phi);
        const R D_3 = Eem.z * (D_1 + qem * cos_phi);
        const R D_4 = Eop.z * (D_1 + qop * cos_phi);
        const R N2 = (Eep.x * (qep - q2om) * D_4 + Eop.x * (q2om - qop) * D_2 + Eop.y * B_1 + Eep.y * B_3);
        roo = -(Eep.x * Eom.z * (q2om - qep) * (qop * cos_phi - D_1) + Eom.x * (q2om + qop) * D_2 + Eom.y * B_1 - Eep.y * B_2) / N2;
        roe = -(-Eom.x * Eop.z * (qop * (qop * cos_phi + K * sin_phi) + q2om * D_1) +
                Eom.z * Eop.x * (qop * (qop * cos_phi - K * sin_phi) + q2om * D_1) + Eop.y * B_2 + Eom.y * B_3) / N2;
        tos = (Eep.x * qep * roe - Eom.x * qop + Eop.x * qop * roo) / q2om;
        top = -(Eom.z * qop - Eom.y * K - (Eep.y * K + Eep.z * qep) * roe - (Eop.y * K + Eop.z * qop) * roo) / D_1;
        reo = (Eem.x * (qem - q2om) * (D_2 + Eep.y * K * cos_phi) + Eep.x * (q2om - qep) * (D_3 + Eem.y * K * cos_phi)) / N2;
        ree = -(Eem.x * (qem - q2om) * D_4 - Eem.x * Eop.y * K * cos_phi * (q2om - qem) + Eem.y * B_3 + Eop.x * (q2om - qop) * D_3) / N2;
        tes = (Eem.x * qem + Eep.x * qep * ree + Eop.x * qop * reo) / q2om;
        tep = -(Eem.z + Eep.z * ree + Eop.z * reo) / cos_phi;
    }
    static void vectors_in_slab(V3<R> I, R ei, R eo, R ee, V3<R> A, V3<R>& Io, V3<R>& Io2, V3<R>& Ie, V3<R>& Ie2, R& e_eff, R& e_eff2) {
        const R K = ei * I.z;
        const R qom = -qo(eo, K);
        const R qep = qe(eo, ee, A, K).x;
        const R qem = qe(eo, ee, A, K).y;
        const V3<R> Eom = E_om(eo, A, K);
        const V3<R> Eep = E_ep(eo, ee, A, K);
        const V3<R> Eem = E_em(eo, ee, A, K);
        Io = Poynting(qom, Eom, K);
        Io2 = Io;
        Io2.y = Io2.y * R(-1);
        Ie = Poynting(qem, Eem, K);
        Ie2 = Poynting(qep, Eep, K);
        const V3<R> We = normalize(V3<R>{R(0), qem, -K});
        const V3<R> We2 = normalize(V3<R>{R(0), qep, -K});
        e_eff = K / o_sqrt(o_max(R(0), R(1) - sqr(We.y)));
        e_eff2 = K / o_sqrt(o_max(R(0), R(1) - sqr(We2.y)));
    }
};

}  // namespace plt_oracle

#include "plt_oracle_bsdf.hpp"
