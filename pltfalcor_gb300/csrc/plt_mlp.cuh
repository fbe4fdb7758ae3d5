// Learned MIS proposal for the non-delta BSDF lobes: a conditional MLP
//   x (16 = wi 3, wavelength, roughness, grating pitch, material class one-hot 8, 2 zero pads)
//   -> 64 -> 64 -> 64 (SiLU) -> 32 = 8 x (logit, mu_x, mu_y, log sigma)
// giving a mixture of 8 isotropic Gaussians over the primary sample (u0, u1) in [0,1)^2 that the
// surface model's direction sampler (Gaussian or fractal surface) maps to wo.  BF16 weights and
// activations, FP32 accumulation on the tensor cores (warp-level mma.sync m16n8k16).  No
// counterpart in the reference: PLTPT samples only the analytic BSDF samplers; the proposal is an
// additional one-sample MIS technique in primary sample space, so the exact BSDF is still evaluated
// on every path and the estimate keeps the analytic tracer's expectation.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cstdint>

namespace pltdev {
namespace mlp {

constexpr int kIn = 16, kHid = 64, kOut = 32, kComp = 8;
// parameter layout (elements): W1 [64][16], W2 [64][64], W3 [64][64], W4 [32][64], b1, b2, b3, b4
constexpr int kW1 = 0, kW2 = kW1 + kHid * kIn, kW3 = kW2 + kHid * kHid, kW4 = kW3 + kHid * kHid;
constexpr int kB1 = kW4 + kOut * kHid, kB2 = kB1 + kHid, kB3 = kB2 + kHid, kB4 = kB3 + kHid;
constexpr int kParams = kB4 + kOut;   // 11488
constexpr float kLogSigmaMin = -6.f, kLogSigmaMax = 2.f;

typedef __nv_bfloat16 bf16;

__device__ __forceinline__ uint32_t packBf(float lo, float hi) {
    __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&h);
}
__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}
__device__ __forceinline__ uint32_t ld2(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }
__device__ __forceinline__ float silu(float z) { return z / (1.f + expf(-z)); }
__device__ __forceinline__ float siluGrad(float z) {
    const float s = 1.f / (1.f + expf(-z));
    return s * (1.f + z * (1.f - s));
}

// D = A (16x16 bf16, row) * B (16x8 bf16, col) + D (fp32)
__device__ __forceinline__ void mma16816(float* d, uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, {%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Y[16 x N] = A[16 x K] * W^T for the 16 rows starting at row r0 of a row-major bf16 activation
// tile (stride sa); W is [N][K] row-major bf16 (stride sw).  `act` is true when A holds
// pre-activations Z and the operand is silu(Z) (rounded to bf16).  acc[nt][*] follows the mma
// C fragment: (g, 2q), (g, 2q+1), (g+8, 2q), (g+8, 2q+1) of column tile nt.
template <int K, int N>
__device__ __forceinline__ void warpForwardTile(const bf16* A, int sa, int r0, bool act, const bf16* W, int sw, float (&acc)[N / 8][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
    for (int kt = 0; kt < K / 16; ++kt) {
        const int c0 = kt * 16 + 2 * q;
        uint32_t a[4];
        const bf16* row0 = A + (r0 + g) * sa;
        const bf16* row1 = A + (r0 + g + 8) * sa;
        if (act) {
            a[0] = packBf(silu(__bfloat162float(row0[c0])), silu(__bfloat162float(row0[c0 + 1])));
            a[1] = packBf(silu(__bfloat162float(row1[c0])), silu(__bfloat162float(row1[c0 + 1])));
            a[2] = packBf(silu(__bfloat162float(row0[c0 + 8])), silu(__bfloat162float(row0[c0 + 9])));
            a[3] = packBf(silu(__bfloat162float(row1[c0 + 8])), silu(__bfloat162float(row1[c0 + 9])));
        } else {
            a[0] = ld2(row0 + c0);
            a[1] = ld2(row1 + c0);
            a[2] = ld2(row0 + c0 + 8);
            a[3] = ld2(row1 + c0 + 8);
        }
#pragma unroll
        for (int nt = 0; nt < N / 8; ++nt) {
            const bf16* w = W + (nt * 8 + g) * sw + c0;
            mma16816(acc[nt], a[0], a[1], a[2], a[3], ld2(w), ld2(w + 8));
        }
    }
}

// Stores acc + bias, rounded to bf16, into rows r0.. of a [rows][stride] pre-activation tile.
template <int N>
__device__ __forceinline__ void storeZ(const float (&acc)[N / 8][4], const float* bias, bf16* Z, int sz, int r0) {
    const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt) {
        const int c = nt * 8 + 2 * q;
        *reinterpret_cast<uint32_t*>(Z + (r0 + g) * sz + c) = packBf(acc[nt][0] + bias[c], acc[nt][1] + bias[c + 1]);
        *reinterpret_cast<uint32_t*>(Z + (r0 + g + 8) * sz + c) = packBf(acc[nt][2] + bias[c], acc[nt][3] + bias[c + 1]);
    }
}
template <int N>
__device__ __forceinline__ void storeOut(const float (&acc)[N / 8][4], const float* bias, float* O, int so, int r0) {
    const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt) {
        const int c = nt * 8 + 2 * q;
        O[(r0 + g) * so + c] = acc[nt][0] + bias[c];
        O[(r0 + g) * so + c + 1] = acc[nt][1] + bias[c + 1];
        O[(r0 + g + 8) * so + c] = acc[nt][2] + bias[c];
        O[(r0 + g + 8) * so + c + 1] = acc[nt][3] + bias[c + 1];
    }
}

// Shared-memory copy of the network (bf16 weights with padded rows, fp32 biases).
constexpr int kSW1 = kIn + 8, kSWH = kHid + 8;   // row strides (elements)
struct SmemNet {
    bf16 w1[kHid * kSW1];
    bf16 w2[kHid * kSWH];
    bf16 w3[kHid * kSWH];
    bf16 w4[kOut * kSWH];
    float b[kHid * 3 + kOut];
};
__device__ __forceinline__ void loadNet(SmemNet& s, const bf16* __restrict__ p) {
    for (int i = threadIdx.x; i < kHid * kIn; i += blockDim.x) s.w1[(i / kIn) * kSW1 + i % kIn] = p[kW1 + i];
    for (int i = threadIdx.x; i < kHid * kHid; i += blockDim.x) {
        s.w2[(i / kHid) * kSWH + i % kHid] = p[kW2 + i];
        s.w3[(i / kHid) * kSWH + i % kHid] = p[kW3 + i];
    }
    for (int i = threadIdx.x; i < kOut * kHid; i += blockDim.x) s.w4[(i / kHid) * kSWH + i % kHid] = p[kW4 + i];
    for (int i = threadIdx.x; i < kHid * 3 + kOut; i += blockDim.x) s.b[i] = __bfloat162float(p[kB1 + i]);
}

// Mixture parameters of one output row: weights (softmax), means, sigmas.
struct Mixture {
    float pi[kComp], mx[kComp], my[kComp], sig[kComp];
};
__device__ __forceinline__ void decodeMixture(const float* out, Mixture& m) {
    float mx = -3.4e38f;
#pragma unroll
    for (int k = 0; k < kComp; ++k) mx = fmaxf(mx, out[4 * k]);
    float sum = 0.f;
#pragma unroll
    for (int k = 0; k < kComp; ++k) {
        m.pi[k] = expf(out[4 * k] - mx);
        sum += m.pi[k];
        m.mx[k] = out[4 * k + 1];
        m.my[k] = out[4 * k + 2];
        m.sig[k] = expf(fminf(fmaxf(out[4 * k + 3], kLogSigmaMin), kLogSigmaMax));
    }
    const float inv = 1.f / sum;
#pragma unroll
    for (int k = 0; k < kComp; ++k) m.pi[k] *= inv;
}
// density at (x, y)
__device__ __forceinline__ float mixtureDensity(const Mixture& m, float x, float y) {
    float p = 0.f;
#pragma unroll
    for (int k = 0; k < kComp; ++k) {
        const float dx = x - m.mx[k], dy = y - m.my[k];
        const float is2 = 1.f / (m.sig[k] * m.sig[k]);
        p += m.pi[k] * (0.159154943091895335769f * is2) * expf(-0.5f * (dx * dx + dy * dy) * is2);
    }
    return p;
}

// ---- inference inside the path tracer ------------------------------------------------------

// Feature row of one query: wi in the shading frame (z > 0), the hero wavelength (nm) and the
// material's (roughness, pitch feature, class, enabled).
__device__ __forceinline__ void featureRow(float wx, float wy, float wz, float wl, float4 mf, float* x) {
    x[0] = wx;
    x[1] = wy;
    x[2] = wz;
    x[3] = (wl - 550.f) * (1.f / 170.f);
    x[4] = mf.x;
    x[5] = mf.y;
    const int cls = (int)mf.z;
#pragma unroll
    for (int c = 0; c < 8; ++c) x[6 + c] = cls == c ? 1.f : 0.f;
    x[14] = x[15] = 0.f;
}

// Forward of the 32 rows of one warp in place in a [32][kSWH] bf16 buffer: inputs in columns
// 0..15 on entry, the 32 fp32 outputs in the first 128 bytes of each row on exit.  Every layer
// reads its 16-row tile completely before the warp overwrites it.
__device__ __forceinline__ void warpForward32InPlace(bf16* buf, const SmemNet& net) {
#pragma unroll 1
    for (int t = 0; t < 2; ++t) {
        const int r = 16 * t;
        float a64[kHid / 8][4], a32[kOut / 8][4];
        warpForwardTile<kIn, kHid>(buf, kSWH, r, false, net.w1, kSW1, a64);
        __syncwarp();
        storeZ<kHid>(a64, net.b, buf, kSWH, r);
        __syncwarp();
        warpForwardTile<kHid, kHid>(buf, kSWH, r, true, net.w2, kSWH, a64);
        __syncwarp();
        storeZ<kHid>(a64, net.b + kHid, buf, kSWH, r);
        __syncwarp();
        warpForwardTile<kHid, kHid>(buf, kSWH, r, true, net.w3, kSWH, a64);
        __syncwarp();
        storeZ<kHid>(a64, net.b + 2 * kHid, buf, kSWH, r);
        __syncwarp();
        warpForwardTile<kHid, kOut>(buf, kSWH, r, true, net.w4, kSWH, a32);
        __syncwarp();
        storeOut<kOut>(a32, net.b + 3 * kHid, reinterpret_cast<float*>(buf), kSWH / 2, r);
        __syncwarp();
    }
}

// A vertex's mixture as the path tracer keeps it: per component (weight, mu_x) and (mu_y, sigma)
// as binary16 pairs (half the registers of the fp32 form); sampling and density use these values.
struct PropMix {
    uint2 c[kComp];
};
__device__ __forceinline__ uint32_t packHalf2(float lo, float hi) {
    return (uint32_t)__half_as_ushort(__float2half_rn(lo)) | ((uint32_t)__half_as_ushort(__float2half_rn(hi)) << 16);
}
__device__ __forceinline__ float halfLo(uint32_t v) { return __half2float(__ushort_as_half((unsigned short)(v & 0xFFFFu))); }
__device__ __forceinline__ float halfHi(uint32_t v) { return __half2float(__ushort_as_half((unsigned short)(v >> 16))); }

__device__ __forceinline__ void packMixture(const float* out, PropMix& pm) {
    Mixture m;
    decodeMixture(out, m);
#pragma unroll
    for (int k = 0; k < kComp; ++k) pm.c[k] = make_uint2(packHalf2(m.pi[k], m.mx[k]), packHalf2(m.my[k], m.sig[k]));
}
// density at (x, y): sum_k (w_k / sum w) N((x, y); mu_k, sigma_k^2 I)
__device__ __forceinline__ float mixtureDensityPacked(const PropMix& pm, float x, float y) {
    float s = 0.f, p = 0.f;
#pragma unroll
    for (int k = 0; k < kComp; ++k) {
        const float w = halfLo(pm.c[k].x), dx = x - halfHi(pm.c[k].x), dy = y - halfLo(pm.c[k].y), sg = halfHi(pm.c[k].y);
        const float is2 = 1.f / (sg * sg);
        s += w;
        p += w * (0.159154943091895335769f * is2) * expf(-0.5f * (dx * dx + dy * dy) * is2);
    }
    return s > 0.f ? p / s : 0.f;
}
// Draws (x, y) from the mixture: a component by u0 over the cumulative weights, then a Box-Muller
// Gaussian step from (u1, u2).
__device__ __forceinline__ void sampleMixturePacked(const PropMix& pm, float u0, float u1, float u2, float& x, float& y) {
    float s = 0.f;
#pragma unroll
    for (int k = 0; k < kComp; ++k) s += halfLo(pm.c[k].x);
    const float t = u0 * s;
    float cum = 0.f, mx = 0.f, my = 0.f, sg = 0.f, lmx = 0.f, lmy = 0.f, lsg = 0.f;
    bool found = false;
#pragma unroll
    for (int k = 0; k < kComp; ++k) {
        const float w = halfLo(pm.c[k].x);
        cum += w;
        if (w > 0.f) { lmx = halfHi(pm.c[k].x); lmy = halfLo(pm.c[k].y); lsg = halfHi(pm.c[k].y); }
        if (!found && t < cum) { found = true; mx = halfHi(pm.c[k].x); my = halfLo(pm.c[k].y); sg = halfHi(pm.c[k].y); }
    }
    if (!found) { mx = lmx; my = lmy; sg = lsg; }
    const float r = sg * sqrtf(-2.f * logf(1.f - u1));
    float sn, cs;
    sincosf(6.28318530717958647692f * u2, &sn, &cs);
    x = mx + r * cs;
    y = my + r * sn;
}

}  // namespace mlp
}  // namespace pltdev
