// Training and batch inference of the learned MIS proposal (plt_mlp.cuh): training samples drawn
// from the exact non-delta BSDF samplers, a fused forward + mixture-NLL + backward kernel (one CTA
// per 128 samples, tensor-core MMAs for every layer and for the weight gradients), Adam on FP32
// master weights with a BF16 copy for the kernels.
#include <algorithm>
#include <cmath>

#include "plt_mlp.cuh"
#include "plt_pt.cuh"

namespace pltdev {
namespace mlp {

constexpr int kRows = 128;                 // samples per CTA (4 warps x 32 rows)
constexpr int kSX = kIn + 8, kSZ = kHid + 8, kSD4 = kOut + 8, kSO = kOut;

// Feature vector of one query (wi in the z >= 0 frame): wi, wavelength, roughness, pitch,
// material class one-hot.  mf = (roughness, pitch feature, class, enabled) of the material.
__device__ __forceinline__ void features(f3 wi, float wl, float4 mf, float* x) { featureRow(wi.x, wi.y, wi.z, wl, mf, x); }

// One training sample per thread: a material among the enabled ones, wi uniform on the upper
// hemisphere (cos >= 0.01), a wavelength in 380-720 nm and a uniform primary sample u that the
// material's exact sampler, restricted to the non-delta lobes, turns into wo.  The target is u; the
// weight is what the path tracer's forward replay multiplies the path by at this vertex: the BSDF
// value (an unpolarised unit beam of 1 mm^2 coherence area at 1 m arriving from wo, leaving towards
// wi) over the sampler's pdf, clamped to 4; 0 when no direction was produced.  The weighted
// likelihood then fits q(u) proportional to the expected contribution of u.
__global__ void __launch_bounds__(128) proposalDataKernel(const DevMaterial* __restrict__ mats, const float4* __restrict__ matFeat,
                                                          const uint2* __restrict__ matProps, const uint32_t* __restrict__ enabled,
                                                          uint32_t nEnabled, const DevProfile* __restrict__ profiles, uint32_t nProfiles,
                                                          uint32_t flags, uint32_t n, uint32_t seed, bf16* __restrict__ x,
                                                          float* __restrict__ target, float* __restrict__ weight) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    SampleGen sg;
    sg.init(i & 0xFFFFu, i >> 16, seed);
    const uint32_t mid = __ldg(enabled + min((uint32_t)(sg.next1D() * (float)nEnabled), nEnabled - 1));
    const float z = 0.01f + 0.99f * sg.next1D();
    const float phi = k2Pi * sg.next1D();
    float sp, cp;
    sincosf(phi, &sp, &cp);
    const float rxy = sqrtf(fmaxf(0.f, 1.f - z * z));
    const f3 wi = mk3(rxy * cp, rxy * sp, z);
    const float wl = 380.f + 340.f * sg.next1D();
    const f2 u = {sg.next1D(), sg.next1D()};
    SD sd;
    sd.posW = mk3(0.f, 0.f, 0.f);
    sd.V = wi;
    sd.N = mk3(0.f, 0.f, 1.f);
    sd.T = mk3(1.f, 0.f, 0.f);
    sd.B = mk3(0.f, 1.f, 0.f);
    sd.faceN = sd.N;
    sd.frontFacing = true;
    const DevMaterial* __restrict__ m = mats + mid;
    const uint32_t type = __ldg(&m->type);
    f3 wo = mk3(0.f, 0.f, 0.f);
    float pdf = 0.f, w = 0.f;
    uint32_t lobe = 0;
    const bool ok = ptSample(m, type, sd, sg, wl, wo, pdf, w, lobe, kLobeNonDelta, mk3(0.f, 0.f, 0.f), u);
    bool valid = ok && pdf > 0.f && isfinite(wo.x) && isfinite(wo.y) && isfinite(wo.z) && (lobe & kLobeDelta) == 0;
    float contrib = 0.f;
    if (valid) {
        // the forward replay's view of the vertex (prepareSD with V towards the light side)
        SD se = sd;
        se.V = wo;
        se.frontFacing = wo.z >= 0.f;
        if (!se.frontFacing && (__ldg(matProps + mid).x & plt::kPropDoubleSided)) se.N = mk3(0.f, 0.f, -1.f);
        DBeam<1> b;
        b.L[0][0] = 1.f;
        b.L[1][0] = b.L[2][0] = b.L[3][0] = 0.f;
        b.wl[0] = wl;
        b.D0 = 1.f; b.D1 = 0.f; b.D2 = 1.f;
        b.r_m = 1.f;
        b.r = -wo;
        b.t = perp_stark(b.r);
        const Ctx c{profiles, nProfiles, flags};
        ptEval<1>(m, type, c, se, wi, lobe, b);
        contrib = b.L[0][0] / pdf;
        valid = isfinite(contrib);
    }
    float f[16];
    features(wi, wl, __ldg(matFeat + mid), f);
#pragma unroll
    for (int c = 0; c < 16; c += 2) *reinterpret_cast<uint32_t*>(x + (size_t)i * kIn + c) = packBf(f[c], f[c + 1]);
    target[2 * (size_t)i] = u.x;
    target[2 * (size_t)i + 1] = u.y;
    weight[i] = valid ? fminf(fmaxf(contrib, 0.f), 4.f) : 0.f;
}

// Mixture negative log-likelihood of one sample and its gradient w.r.t. the 32 outputs.
__device__ __forceinline__ float mixtureNllGrad(const float* out, float tx, float ty, float w, float* d) {
    if (!(w > 0.f)) {
#pragma unroll
        for (int j = 0; j < kOut; ++j) d[j] = 0.f;
        return 0.f;
    }
    float lmax = -3.4e38f;
#pragma unroll
    for (int k = 0; k < kComp; ++k) lmax = fmaxf(lmax, out[4 * k]);
    float lsum = 0.f;
#pragma unroll
    for (int k = 0; k < kComp; ++k) lsum += expf(out[4 * k] - lmax);
    const float lse = lmax + logf(lsum);
    float a[kComp], d2s[kComp];
    float amax = -3.4e38f;
#pragma unroll
    for (int k = 0; k < kComp; ++k) {
        const float s = fminf(fmaxf(out[4 * k + 3], kLogSigmaMin), kLogSigmaMax);
        const float is2 = expf(-2.f * s);
        const float dx = tx - out[4 * k + 1], dy = ty - out[4 * k + 2];
        d2s[k] = (dx * dx + dy * dy) * is2;
        a[k] = (out[4 * k] - lse) - 0.5f * d2s[k] - 2.f * s - 1.83787706640934548356f;   // log(2 pi)
        amax = fmaxf(amax, a[k]);
    }
    float asum = 0.f;
#pragma unroll
    for (int k = 0; k < kComp; ++k) asum += expf(a[k] - amax);
    const float lq = amax + logf(asum);
#pragma unroll
    for (int k = 0; k < kComp; ++k) {
        const float r = expf(a[k] - lq);
        const float pik = expf(out[4 * k] - lse);
        const float s = out[4 * k + 3];
        const float is2 = expf(-2.f * fminf(fmaxf(s, kLogSigmaMin), kLogSigmaMax));
        d[4 * k] = -w * (r - pik);
        d[4 * k + 1] = -w * r * (tx - out[4 * k + 1]) * is2;
        d[4 * k + 2] = -w * r * (ty - out[4 * k + 2]) * is2;
        d[4 * k + 3] = (s > kLogSigmaMin && s < kLogSigmaMax) ? -w * r * (d2s[k] - 2.f) : 0.f;
    }
    return -w * lq;
}

// dH[16 x N] = D[16 x K] * W[K][N] (W row-major [K][N], stride sw): backward through a layer.
template <int K, int N>
__device__ __forceinline__ void warpBackTile(const bf16* D, int sd, int r0, const bf16* W, int sw, float (&acc)[N / 8][4]) {
    const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt) acc[nt][0] = acc[nt][1] = acc[nt][2] = acc[nt][3] = 0.f;
#pragma unroll
    for (int kt = 0; kt < K / 16; ++kt) {
        const int c0 = kt * 16 + 2 * q;
        const bf16* row0 = D + (r0 + g) * sd;
        const bf16* row1 = D + (r0 + g + 8) * sd;
        const uint32_t a0 = ld2(row0 + c0), a1 = ld2(row1 + c0), a2 = ld2(row0 + c0 + 8), a3 = ld2(row1 + c0 + 8);
#pragma unroll
        for (int nt = 0; nt < N / 8; ++nt) {
            const int nn = nt * 8 + g;
            const uint32_t b0 = pack2(W[c0 * sw + nn], W[(c0 + 1) * sw + nn]);
            const uint32_t b1 = pack2(W[(c0 + 8) * sw + nn], W[(c0 + 9) * sw + nn]);
            mma16816(acc[nt], a0, a1, a2, a3, b0, b1);
        }
    }
}
// D_out = acc * silu'(Z), rounded to bf16
template <int N>
__device__ __forceinline__ void storeDZ(const float (&acc)[N / 8][4], const bf16* Z, int sz, bf16* D, int sd, int r0) {
    const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
#pragma unroll
    for (int nt = 0; nt < N / 8; ++nt) {
        const int c = nt * 8 + 2 * q;
        const bf16* z0 = Z + (r0 + g) * sz + c;
        const bf16* z1 = Z + (r0 + g + 8) * sz + c;
        *reinterpret_cast<uint32_t*>(D + (r0 + g) * sd + c) =
            packBf(acc[nt][0] * siluGrad(__bfloat162float(z0[0])), acc[nt][1] * siluGrad(__bfloat162float(z0[1])));
        *reinterpret_cast<uint32_t*>(D + (r0 + g + 8) * sd + c) =
            packBf(acc[nt][2] * siluGrad(__bfloat162float(z1[0])), acc[nt][3] * siluGrad(__bfloat162float(z1[1])));
    }
}
// One 16 x 8 tile of dW[o][i] = sum_s D[s][o] * X[s][i] over the CTA's 128 samples; X is silu(Z)
// when `act`.  The result, scaled, is added to the global gradient.
__device__ __forceinline__ void weightGradTile(const bf16* D, int sd, const bf16* X, int sx, bool act, int m0, int n0, int fanIn,
                                               float* gW, float scale) {
    const int lane = threadIdx.x & 31, g = lane >> 2, q = lane & 3;
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
    auto xv = [&](int s, int i) {
        const float v = __bfloat162float(X[s * sx + i]);
        return act ? __float2bfloat16_rn(silu(v)) : X[s * sx + i];
    };
#pragma unroll
    for (int kt = 0; kt < kRows / 16; ++kt) {
        const int s0 = kt * 16 + 2 * q;
        const uint32_t a0 = pack2(D[s0 * sd + m0 + g], D[(s0 + 1) * sd + m0 + g]);
        const uint32_t a1 = pack2(D[s0 * sd + m0 + g + 8], D[(s0 + 1) * sd + m0 + g + 8]);
        const uint32_t a2 = pack2(D[(s0 + 8) * sd + m0 + g], D[(s0 + 9) * sd + m0 + g]);
        const uint32_t a3 = pack2(D[(s0 + 8) * sd + m0 + g + 8], D[(s0 + 9) * sd + m0 + g + 8]);
        const uint32_t b0 = pack2(xv(s0, n0 + g), xv(s0 + 1, n0 + g));
        const uint32_t b1 = pack2(xv(s0 + 8, n0 + g), xv(s0 + 9, n0 + g));
        mma16816(acc, a0, a1, a2, a3, b0, b1);
    }
    const int c = n0 + 2 * q;
    atomicAdd(gW + (m0 + g) * fanIn + c, acc[0] * scale);
    atomicAdd(gW + (m0 + g) * fanIn + c + 1, acc[1] * scale);
    atomicAdd(gW + (m0 + g + 8) * fanIn + c, acc[2] * scale);
    atomicAdd(gW + (m0 + g + 8) * fanIn + c + 1, acc[3] * scale);
}

struct GradSmem {
    SmemNet net;
    bf16 x[kRows * kSX];
    bf16 z1[kRows * kSZ], z2[kRows * kSZ], z3[kRows * kSZ];
    bf16 d4[kRows * kSD4];
    bf16 d3[kRows * kSZ], d2[kRows * kSZ], d1[kRows * kSZ];
    float out[kRows * kSO];
    float tgt[kRows * 2], w[kRows];
};

// Forward of the 32 rows of warp `warp` (rows r0..r0+31) up to the 32 outputs.
__device__ __forceinline__ void forwardRows(GradSmem& s, int r0) {
    for (int t = 0; t < 2; ++t) {
        const int r = r0 + 16 * t;
        float a64[8][4], a32[4][4];
        warpForwardTile<kIn, kHid>(s.x, kSX, r, false, s.net.w1, kSW1, a64);
        storeZ<kHid>(a64, s.net.b, s.z1, kSZ, r);
        __syncwarp();
        warpForwardTile<kHid, kHid>(s.z1, kSZ, r, true, s.net.w2, kSWH, a64);
        storeZ<kHid>(a64, s.net.b + kHid, s.z2, kSZ, r);
        __syncwarp();
        warpForwardTile<kHid, kHid>(s.z2, kSZ, r, true, s.net.w3, kSWH, a64);
        storeZ<kHid>(a64, s.net.b + 2 * kHid, s.z3, kSZ, r);
        __syncwarp();
        warpForwardTile<kHid, kOut>(s.z3, kSZ, r, true, s.net.w4, kSWH, a32);
        storeOut<kOut>(a32, s.net.b + 3 * kHid, s.out, kSO, r);
        __syncwarp();
    }
}

// Gradient of the mean weighted mixture NLL over the batch w.r.t. all parameters (added into
// grad, which the caller zeroes), and the loss (added into loss[0]).  invN = 1 / batch size.
__global__ void __launch_bounds__(128) proposalGradKernel(const bf16* __restrict__ params, const bf16* __restrict__ x,
                                                          const float* __restrict__ target, const float* __restrict__ weight, uint32_t n,
                                                          float invN, float* __restrict__ grad, float* __restrict__ loss) {
    extern __shared__ __align__(16) unsigned char smemRaw[];
    GradSmem& s = *reinterpret_cast<GradSmem*>(smemRaw);
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t base = blockIdx.x * kRows;
    loadNet(s.net, params);
    for (int i = tid; i < kRows * kIn / 2; i += blockDim.x) {
        const int r = i / (kIn / 2), c = 2 * (i % (kIn / 2));
        const uint32_t v = (base + r < n) ? *reinterpret_cast<const uint32_t*>(x + (size_t)(base + r) * kIn + c) : 0u;
        *reinterpret_cast<uint32_t*>(s.x + r * kSX + c) = v;
    }
    {
        const bool in = base + tid < n;
        s.tgt[2 * tid] = in ? target[2 * (size_t)(base + tid)] : 0.f;
        s.tgt[2 * tid + 1] = in ? target[2 * (size_t)(base + tid) + 1] : 0.f;
        s.w[tid] = in ? weight[base + tid] : 0.f;
    }
    __syncthreads();
    const int r0 = warp * 32;
    forwardRows(s, r0);
    // loss and output gradient, one row per thread (row tid belongs to this thread's warp)
    float d[kOut];
    const float l = mixtureNllGrad(s.out + tid * kSO, s.tgt[2 * tid], s.tgt[2 * tid + 1], s.w[tid], d);
#pragma unroll
    for (int j = 0; j < kOut; j += 2) *reinterpret_cast<uint32_t*>(s.d4 + tid * kSD4 + j) = packBf(d[j], d[j + 1]);
    float lsum = l;
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xFFFFFFFFu, lsum, o);
    if ((tid & 31) == 0) atomicAdd(loss, lsum * invN);
    __syncwarp();
    // backward through the layers, rows of this warp
    for (int t = 0; t < 2; ++t) {
        const int r = r0 + 16 * t;
        float a64[8][4];
        warpBackTile<kOut, kHid>(s.d4, kSD4, r, s.net.w4, kSWH, a64);
        storeDZ<kHid>(a64, s.z3, kSZ, s.d3, kSZ, r);
        __syncwarp();
        warpBackTile<kHid, kHid>(s.d3, kSZ, r, s.net.w3, kSWH, a64);
        storeDZ<kHid>(a64, s.z2, kSZ, s.d2, kSZ, r);
        __syncwarp();
        warpBackTile<kHid, kHid>(s.d2, kSZ, r, s.net.w2, kSWH, a64);
        storeDZ<kHid>(a64, s.z1, kSZ, s.d1, kSZ, r);
        __syncwarp();
    }
    __syncthreads();
    // weight gradients: 88 tiles of 16 x 8 over the four layers, spread over the warps
    for (int tile = warp; tile < 88; tile += 4) {
        if (tile < 16) {            // W4 [32][64] = D4^T H3
            weightGradTile(s.d4, kSD4, s.z3, kSZ, true, (tile / 8) * 16, (tile % 8) * 8, kHid, grad + kW4, invN);
        } else if (tile < 48) {     // W3 [64][64] = D3^T H2
            const int t = tile - 16;
            weightGradTile(s.d3, kSZ, s.z2, kSZ, true, (t / 8) * 16, (t % 8) * 8, kHid, grad + kW3, invN);
        } else if (tile < 80) {     // W2 [64][64] = D2^T H1
            const int t = tile - 48;
            weightGradTile(s.d2, kSZ, s.z1, kSZ, true, (t / 8) * 16, (t % 8) * 8, kHid, grad + kW2, invN);
        } else {                    // W1 [64][16] = D1^T X
            const int t = tile - 80;
            weightGradTile(s.d1, kSZ, s.x, kSX, false, (t / 2) * 16, (t % 2) * 8, kIn, grad + kW1, invN);
        }
    }
    // bias gradients: column sums
    for (int c = tid; c < 3 * kHid + kOut; c += blockDim.x) {
        const bf16* D;
        int sd, col, off;
        if (c < kHid) { D = s.d1; sd = kSZ; col = c; off = kB1; }
        else if (c < 2 * kHid) { D = s.d2; sd = kSZ; col = c - kHid; off = kB2; }
        else if (c < 3 * kHid) { D = s.d3; sd = kSZ; col = c - 2 * kHid; off = kB3; }
        else { D = s.d4; sd = kSD4; col = c - 3 * kHid; off = kB4; }
        float acc = 0.f;
        for (int r = 0; r < kRows; ++r) acc += __bfloat162float(D[r * sd + col]);
        atomicAdd(grad + off + col, acc * invN);
    }
}

// Batch inference: out[n][32] (fp32) for feature rows x[n][16] (bf16).
__global__ void __launch_bounds__(128) proposalForwardKernel(const bf16* __restrict__ params, const bf16* __restrict__ x, uint32_t n,
                                                             float* __restrict__ out) {
    extern __shared__ __align__(16) unsigned char smemRaw[];
    GradSmem& s = *reinterpret_cast<GradSmem*>(smemRaw);
    const int tid = threadIdx.x, warp = tid >> 5;
    const uint32_t base = blockIdx.x * kRows;
    loadNet(s.net, params);
    for (int i = tid; i < kRows * kIn / 2; i += blockDim.x) {
        const int r = i / (kIn / 2), c = 2 * (i % (kIn / 2));
        const uint32_t v = (base + r < n) ? *reinterpret_cast<const uint32_t*>(x + (size_t)(base + r) * kIn + c) : 0u;
        *reinterpret_cast<uint32_t*>(s.x + r * kSX + c) = v;
    }
    __syncthreads();
    forwardRows(s, warp * 32);
    __syncthreads();
    for (int i = tid; i < kRows * kOut; i += blockDim.x) {
        const int r = i / kOut, c = i % kOut;
        if (base + r < n) out[(size_t)(base + r) * kOut + c] = s.out[r * kSO + c];
    }
}

// Adam (Kingma & Ba 2015) on the FP32 master weights; writes the BF16 copy the kernels read.
__global__ void proposalAdamKernel(float* __restrict__ p, float* __restrict__ m, float* __restrict__ v, const float* __restrict__ g,
                                   bf16* __restrict__ pb, float lr, float b1, float b2, float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    p[i] = pi;
    pb[i] = __float2bfloat16_rn(pi);
}

__global__ void toBf16Kernel(const float* __restrict__ p, bf16* __restrict__ pb, int count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < count) pb[i] = __float2bfloat16_rn(p[i]);
}

}  // namespace mlp
}  // namespace pltdev

namespace plt {

using pltdev::mlp::bf16;

static cudaError_t gradSmemAttr(const void* fn) {
    return cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(pltdev::mlp::GradSmem));
}

cudaError_t launchProposalData(const pltdev::DevMaterial* mats, const float4* matFeat, const uint2* matProps, const uint32_t* enabled,
                               uint32_t nEnabled, const pltdev::DevProfile* profiles, uint32_t nProfiles, uint32_t flags, uint32_t n,
                               uint32_t seed, void* x, float* target, float* weight, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    pltdev::mlp::proposalDataKernel<<<(n + 127) / 128, 128, 0, stream>>>(mats, matFeat, matProps, enabled, nEnabled, profiles, nProfiles,
                                                                         flags, n, seed, static_cast<bf16*>(x), target, weight);
    return cudaGetLastError();
}

cudaError_t launchProposalGrad(const void* params, const void* x, const float* target, const float* weight, uint32_t n, float* grad,
                               float* loss, cudaStream_t stream) {
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = gradSmemAttr((const void*)pltdev::mlp::proposalGradKernel);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    cudaError_t e = cudaMemsetAsync(grad, 0, sizeof(float) * pltdev::mlp::kParams, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(loss, 0, sizeof(float), stream);
    if (e != cudaSuccess) return e;
    if (n == 0) return cudaSuccess;
    pltdev::mlp::proposalGradKernel<<<(n + 127) / 128, 128, sizeof(pltdev::mlp::GradSmem), stream>>>(
        static_cast<const bf16*>(params), static_cast<const bf16*>(x), target, weight, n, 1.f / (float)n, grad, loss);
    return cudaGetLastError();
}

cudaError_t launchProposalForward(const void* params, const void* x, uint32_t n, float* out, cudaStream_t stream) {
    static bool attr = false;
    if (!attr) {
        const cudaError_t e = gradSmemAttr((const void*)pltdev::mlp::proposalForwardKernel);
        if (e != cudaSuccess) return e;
        attr = true;
    }
    if (n == 0) return cudaSuccess;
    pltdev::mlp::proposalForwardKernel<<<(n + 127) / 128, 128, sizeof(pltdev::mlp::GradSmem), stream>>>(
        static_cast<const bf16*>(params), static_cast<const bf16*>(x), n, out);
    return cudaGetLastError();
}

cudaError_t launchProposalAdam(float* p, float* m, float* v, const float* g, void* pb, float lr, uint32_t step, cudaStream_t stream) {
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
    pltdev::mlp::proposalAdamKernel<<<(pltdev::mlp::kParams + 255) / 256, 256, 0, stream>>>(p, m, v, g, static_cast<bf16*>(pb), lr, b1, b2,
                                                                                             1e-8f, c1, c2);
    return cudaGetLastError();
}

cudaError_t launchProposalToBf16(const float* p, void* pb, cudaStream_t stream) {
    pltdev::mlp::toBf16Kernel<<<(pltdev::mlp::kParams + 255) / 256, 256, 0, stream>>>(p, static_cast<bf16*>(pb), pltdev::mlp::kParams);
    return cudaGetLastError();
}

}  // namespace plt
