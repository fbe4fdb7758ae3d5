// ORACLE -- test infrastructure only.  The learned MIS proposal's network on the CPU (shared by
// the network oracle, plt_oracle_mlp.cpp, and the path-tracing oracle, plt_oracle_pt.cpp): the
// 16 -> 64 -> 64 -> 64 -> 32 SiLU MLP of pltfalcor_gb300/csrc/plt_mlp.cuh in double with optional
// BF16 rounding of every stored value, and the path tracer's use of its output (feature rows,
// the mixture packed as binary16, its density and its sampling).  No counterpart in the reference.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "plt_oracle_geom.hpp"

namespace plt_oracle_mlp {

constexpr int kIn = 16, kHid = 64, kOut = 32, kComp = 8;
constexpr int kW1 = 0, kW2 = kW1 + kHid * kIn, kW3 = kW2 + kHid * kHid, kW4 = kW3 + kHid * kHid;
constexpr int kB1 = kW4 + kOut * kHid, kB2 = kB1 + kHid, kB3 = kB2 + kHid, kB4 = kB3 + kHid;
constexpr int kParams = kB4 + kOut;
constexpr double kLogSigmaMin = -6.0, kLogSigmaMax = 2.0;

inline float bf16Round(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7F800000u) == 0x7F800000u) return f;
    u += 0x7FFFu + ((u >> 16) & 1u);
    u &= 0xFFFF0000u;
    std::memcpy(&f, &u, 4);
    return f;
}
inline float bf16Bits(uint16_t h) {
    const uint32_t u = (uint32_t)h << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

struct Net {
    bool round;
    std::vector<double> p;
    double q(double v) const { return round ? (double)bf16Round((float)v) : v; }
    double silu(double z) const { return round ? (double)((float)z / (1.f + std::exp(-(float)z))) : z / (1.0 + std::exp(-z)); }
    double siluGrad(double z) const {
        if (round) {
            const float s = 1.f / (1.f + std::exp(-(float)z));
            return (double)(s * (1.f + (float)z * (1.f - s)));
        }
        const double s = 1.0 / (1.0 + std::exp(-z));
        return s * (1.0 + z * (1.0 - s));
    }
    explicit Net(const float* params, bool r) : round(r), p(kParams) {
        for (int i = 0; i < kParams; ++i) p[i] = round ? (double)bf16Round(params[i]) : (double)params[i];
    }
    // forward of one row: Z1..Z3 (stored values) and outputs
    void forward(const double* x, double* z1, double* z2, double* z3, double* out) const {
        for (int o = 0; o < kHid; ++o) {
            double a = 0.0;
            for (int i = 0; i < kIn; ++i) a += x[i] * p[kW1 + o * kIn + i];
            z1[o] = q(a + p[kB1 + o]);
        }
        double h[kHid];
        for (int i = 0; i < kHid; ++i) h[i] = q(silu(z1[i]));
        for (int o = 0; o < kHid; ++o) {
            double a = 0.0;
            for (int i = 0; i < kHid; ++i) a += h[i] * p[kW2 + o * kHid + i];
            z2[o] = q(a + p[kB2 + o]);
        }
        for (int i = 0; i < kHid; ++i) h[i] = q(silu(z2[i]));
        for (int o = 0; o < kHid; ++o) {
            double a = 0.0;
            for (int i = 0; i < kHid; ++i) a += h[i] * p[kW3 + o * kHid + i];
            z3[o] = q(a + p[kB3 + o]);
        }
        for (int i = 0; i < kHid; ++i) h[i] = q(silu(z3[i]));
        for (int o = 0; o < kOut; ++o) {
            double a = 0.0;
            for (int i = 0; i < kHid; ++i) a += h[i] * p[kW4 + o * kHid + i];
            out[o] = round ? (double)(float)(a + p[kB4 + o]) : a + p[kB4 + o];
        }
    }
};

// Feature row of one path-tracer query (plt_mlp.cuh featureRow): wi in the shading frame, hero
// wavelength, the material's (roughness, pitch feature, class); rounded to bf16 as the GPU stores it.
inline void featureRow(float wx, float wy, float wz, float wl, const float mf[4], double* x) {
    float f[kIn];
    f[0] = wx;
    f[1] = wy;
    f[2] = wz;
    f[3] = (wl - 550.f) * (1.f / 170.f);
    f[4] = mf[0];
    f[5] = mf[1];
    const int cls = (int)mf[2];
    for (int c = 0; c < 8; ++c) f[6 + c] = cls == c ? 1.f : 0.f;
    f[14] = f[15] = 0.f;
    for (int i = 0; i < kIn; ++i) x[i] = (double)bf16Round(f[i]);
}

// Packed mixture (plt_mlp.cuh PropMix): per component binary16 (weight, mu_x, mu_y, sigma).
struct PackedMix {
    float w[kComp], mx[kComp], my[kComp], sig[kComp];
};
inline float roundHalf(float v) {
    const uint16_t h = plt_oracle::geom::floatToHalfRne(v);
    const uint32_t sign = (uint32_t)(h & 0x8000u) << 16;
    uint32_t e = (h >> 10) & 0x1Fu, m = h & 0x3FFu, bits;
    if (e == 0) {
        if (m == 0) bits = sign;
        else {
            int k = -1;
            do { ++k; m <<= 1; } while ((m & 0x400u) == 0);
            bits = sign | ((uint32_t)(127 - 15 - k) << 23) | ((m & 0x3FFu) << 13);
        }
    } else if (e == 31) {
        bits = sign | 0x7F800000u | (m << 13);
    } else {
        bits = sign | ((e - 15 + 127) << 23) | (m << 13);
    }
    float f;
    std::memcpy(&f, &bits, 4);
    return f;
}
// decodeMixture (softmax weights, clamped log sigma) in float, then binary16 rounding
inline PackedMix packMixture(const double* out) {
    float o[kOut];
    for (int j = 0; j < kOut; ++j) o[j] = (float)out[j];
    float mx = -3.4e38f;
    for (int k = 0; k < kComp; ++k) mx = std::fmax(mx, o[4 * k]);
    float pi[kComp], sum = 0.f;
    for (int k = 0; k < kComp; ++k) {
        pi[k] = std::exp(o[4 * k] - mx);
        sum += pi[k];
    }
    const float inv = 1.f / sum;
    PackedMix pm;
    for (int k = 0; k < kComp; ++k) {
        pm.w[k] = roundHalf(pi[k] * inv);
        pm.mx[k] = roundHalf(o[4 * k + 1]);
        pm.my[k] = roundHalf(o[4 * k + 2]);
        pm.sig[k] = roundHalf(std::exp(std::fmin(std::fmax(o[4 * k + 3], (float)kLogSigmaMin), (float)kLogSigmaMax)));
    }
    return pm;
}
// density at (x, y), sum_k (w_k / sum w) N((x, y); mu_k, sigma_k^2 I)
inline float mixtureDensity(const PackedMix& pm, float x, float y) {
    float s = 0.f, p = 0.f;
    for (int k = 0; k < kComp; ++k) {
        const float dx = x - pm.mx[k], dy = y - pm.my[k];
        const float is2 = 1.f / (pm.sig[k] * pm.sig[k]);
        s += pm.w[k];
        p += pm.w[k] * (0.159154943091895335769f * is2) * std::exp(-0.5f * (dx * dx + dy * dy) * is2);
    }
    return s > 0.f ? p / s : 0.f;
}
// a component by u0 over the cumulative weights, then a Box-Muller step from (u1, u2)
inline void sampleMixture(const PackedMix& pm, float u0, float u1, float u2, float& x, float& y) {
    float s = 0.f;
    for (int k = 0; k < kComp; ++k) s += pm.w[k];
    const float t = u0 * s;
    float cum = 0.f;
    int sel = -1, last = 0;
    for (int k = 0; k < kComp; ++k) {
        cum += pm.w[k];
        if (pm.w[k] > 0.f) last = k;
        if (sel < 0 && t < cum) sel = k;
    }
    if (sel < 0) sel = last;
    const float r = pm.sig[sel] * std::sqrt(-2.f * std::log(1.f - u1));
    const float a = 6.28318530717958647692f * u2;
    x = pm.mx[sel] + r * std::cos(a);
    y = pm.my[sel] + r * std::sin(a);
}

}  // namespace plt_oracle_mlp
