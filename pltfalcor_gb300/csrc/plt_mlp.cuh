// Learned MIS proposal for the non-delta BSDF lobes: a conditional MLP
//   x (16 = wi 3, wavelength, roughness, grating pitch, material class one-hot 8, 2 zero pads)
//   -> 64 -> 64 -> 64 (SiLU) -> 32 = 8 x (logit, mu_x, mu_y, log sigma)
// giving a mixture of 8 isotropic Gaussians on the projected hemisphere (the unit disk of wo.xy in
// the shading frame).  BF16 weights and activations, FP32 accumulation on the tensor cores
// (warp-level mma.sync m16n8k16).  No counterpart in the reference: PLTPT samples only the
// analytic BSDF samplers; the proposal is an additional one-sample MIS technique, so the exact
// BSDF is still evaluated on every path and the estimate stays unbiased.
#pragma once

#include <cuda_bf16.h>
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
// density on the disk at (x, y)
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

}  // namespace mlp
}  // namespace pltdev
