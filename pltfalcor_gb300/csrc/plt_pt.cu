// PLTPT render pass: frame set-up, the per-segment sample wavefront and the launch sequence of one
// frame (PLTPT::execute, RenderPasses/PLTPT/PLTPT.cpp:357-499 in ssteinberg/PLTFalcor, without the
// tiling, which only bounds the reference's bounce-buffer memory).
#include <algorithm>

#define PLT_PT_SAMPLE_PASS
#include "plt_nvtx.h"
#include "plt_pt.cuh"

namespace pltdev {
__global__ void ptLenCountKernel(const PtParams P);
__global__ void ptLenPrefixKernel(const PtParams P);
__global__ void ptLenScatterKernel(const PtParams P, uint32_t* __restrict__ order);
}  // namespace pltdev

namespace plt {

// the analytic tracer's segment kernel (PLT_BOUNCE_PHASED selects the learned kernel's phased
// structure without the network, for comparison)
#ifdef PLT_BOUNCE_PHASED
static void (*const kPlainBounce)(const PtParams, uint32_t) = pltdev::ptBounceKernel<false>;
#else
static void (*const kPlainBounce)(const PtParams, uint32_t) = pltdev::ptBounceAnalyticKernel;
#endif

// One wave of one frame: the queue counters, the path initialisation, maxBounces + 1 segment
// launches over the compacted queues, then the solve pass and its manifold-walk wavefront.
cudaError_t launchRenderFrame(const PtParams& p, const PtLaunch& L, int numSMs, cudaStream_t stream) {
    if (p.nWave == 0) return cudaSuccess;
    // queue lengths, the manifold-walk count, the solve-order key histogram and its cursors, the
    // walk-order keys, the replay count, the replay-order keys and the replay kernel's work counter,
    // the segments' shading-order keys and work counters
    cudaError_t e = cudaMemsetAsync(p.qcount, 0, sizeof(uint32_t) * ((p.maxBounces + 1) * (1 + 2 * kSolveKeysPerLength) + 2 + 32 + 1 +
                                                                      2 * kReplayKeys + 1 + kSegSortWords * (p.maxBounces + 1)), stream);
    if (e != cudaSuccess) return e;
    // shared memory of the learned variant: the network and one 32-row activation tile per warp
    constexpr size_t kLearnedSmem = sizeof(pltdev::mlp::SmemNet) + 4 * 32 * pltdev::mlp::kSWH * sizeof(pltdev::mlp::bf16);
    static int bpsInit = -1, bpsBounce = -1, bpsLearned = -1, bpsSegTrace = -1;
    const uint32_t gridS = std::min<uint32_t>((p.nWave + 255) / 256, (uint32_t)numSMs * 2);
    if (bpsBounce < 0) {
        int b = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, pltdev::ptSegTraceKernel, 128, 0);
        bpsSegTrace = b > 0 ? b : 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kPlainBounce, 128, 0);
        bpsBounce = b > 0 ? b : 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, pltdev::ptBounceKernel<true>, 128, kLearnedSmem);
        bpsLearned = b > 0 ? b : 1;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, pltdev::ptInitKernel, 128, 0);
        bpsInit = b > 0 ? b : 1;
    }
    auto blocks = [&](int occ, uint32_t want) { return (uint32_t)numSMs * (want ? std::min<uint32_t>(want, (uint32_t)occ) : (uint32_t)occ); };
    const uint32_t need = (p.nWave + 127) / 128;
    {
        const NvtxRange r("pt_init");
        pltdev::ptInitKernel<<<std::min<uint32_t>(need, blocks(bpsInit, 0)), 128, 0, stream>>>(p);
    }
    const NvtxRange rSample("pt_segments");
    // each segment: its closest hits traced with dynamic fetch (and counted by material type), the
    // queue slots sorted by that type, then the segment kernel shades them in that order
    const uint32_t gridT = std::min<uint32_t>(need, blocks(bpsSegTrace, 0));
    if (p.opt & kPtLearned) {
        const uint32_t gridB = std::min<uint32_t>(need, blocks(bpsLearned, L.segBlocksPerSM));
        for (uint32_t it = 0; it <= p.maxBounces; ++it) {
            if (p.segPrim) pltdev::ptSegTraceKernel<<<gridT, 128, 0, stream>>>(p, it);
            if (p.segPrim && p.segOrder) pltdev::ptSegScatterKernel<<<gridS, 256, 0, stream>>>(p, it);
            pltdev::ptBounceKernel<true><<<gridB, 128, kLearnedSmem, stream>>>(p, it);
        }
    } else {
        const uint32_t gridB = std::min<uint32_t>(need, blocks(bpsBounce, L.segBlocksPerSM));
        for (uint32_t it = 0; it <= p.maxBounces; ++it) {
            if (p.segPrim) pltdev::ptSegTraceKernel<<<gridT, 128, 0, stream>>>(p, it);
            if (p.segPrim && p.segOrder) pltdev::ptSegScatterKernel<<<gridS, 256, 0, stream>>>(p, it);
            kPlainBounce<<<gridB, 128, 0, stream>>>(p, it);
        }
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const NvtxRange rSolve("pt_solve");
    PtParams q = p;
    q.order = nullptr;
    // path_order 0: sort waves of at least 2^18 paths (small waves are latency-bound and keep the
    // pixel order's coherence); 1: never; 2: always
    const bool sort = L.noLengthSort == 2u || (L.noLengthSort == 0u && p.nWave >= (1u << 18));
    if (sort) {   // the segment queues are free again: queue0 takes the solve order
        const uint32_t grid = std::min<uint32_t>((p.nWave + 255) / 256, (uint32_t)numSMs * 4);
        pltdev::ptLenCountKernel<<<grid, 256, 0, stream>>>(p);
        pltdev::ptLenPrefixKernel<<<1, 32, 0, stream>>>(p);
        pltdev::ptLenScatterKernel<<<grid, 256, 0, stream>>>(p, p.queue0);
        q.order = p.queue0;
    }
    switch (p.hwss) {
    case 1: return pltdev::launchSolveH<1>(q, L, numSMs, stream);
    case 2: return pltdev::launchSolveH<2>(q, L, numSMs, stream);
    case 3: return pltdev::launchSolveH<3>(q, L, numSMs, stream);
    case 4: return pltdev::launchSolveH<4>(q, L, numSMs, stream);
    case 8: return pltdev::launchSolveH<8>(q, L, numSMs, stream);
    default: return cudaErrorInvalidValue;
    }
}

}  // namespace plt

namespace pltdev {

// The mean of the accumulated frames into each view's output image.
__global__ void ptResolveKernel(const PtParams P, double inv) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < P.nTotal; i += gridDim.x * blockDim.x) {
        const PtScene& S = P.scenes[sceneOf(P, i)];
        float* out = S.out + 4 * (size_t)(i - S.pixelBase);
        out[0] = (float)(P.accum[3 * (size_t)i] * inv);
        out[1] = (float)(P.accum[3 * (size_t)i + 1] * inv);
        out[2] = (float)(P.accum[3 * (size_t)i + 2] * inv);
        out[3] = 1.f;
    }
}

// Solve-pass order of a wave's paths: a counting sort by (path length, material type of the first
// hit), longest first, so that the lanes of a warp replay paths of similar length whose first
// vertex (evaluated by every replay of the path) runs the same material code.  Pass 1 counts the
// keys; pass 2 gives every block a contiguous range of paths, reserves its share of each key's
// slots and scatters.
constexpr uint32_t kSortTypes = plt::kSolveKeysPerLength;
constexpr uint32_t kMaxKeys = 65 * kSortTypes;   // max_bounces <= 64
// second-hit material groups: diffuse-like, dielectric, conductor and coated, grated and layered
__device__ __forceinline__ uint32_t secondGroup(uint32_t t) {
    return (t == kMatDiffuse || t == kMatOpaqueDielectric) ? 0u : (t == kMatDielectric || t == kMatThin) ? 1u
         : (t == kMatConductor || t == kMatCoatedConductor || t == kMatCoatedOpaque) ? 2u : 3u;
}
__device__ __forceinline__ uint32_t solveKey(const PtParams& P, uint32_t i) {
    const uint32_t len = min(P.plen[i], P.maxBounces);
    const uint32_t prim = P.bPrim[i];   // record 0
    uint32_t type = 0, g1 = 0;
    if (prim < P.nTris) type = min(__ldg(&P.mats[__ldg(P.triMat + prim)].type), 15u);
    if (len >= 1) {
        const uint32_t prim1 = P.bPrim[P.npix + i];   // record 1
        if (prim1 < P.nTris) g1 = secondGroup(__ldg(&P.mats[__ldg(P.triMat + prim1)].type));
    }
    // keys in solve order: longer paths first, then by first-hit type, then second-hit group
    return ((P.maxBounces - len) * 16u + type) * 4u + g1;
}
__global__ void __launch_bounds__(256) ptLenCountKernel(const PtParams P) {
    __shared__ uint32_t h[kMaxKeys];
    const uint32_t nk = (P.maxBounces + 1) * kSortTypes;
    for (uint32_t b = threadIdx.x; b < nk; b += blockDim.x) h[b] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < P.nWave; i += gridDim.x * blockDim.x) atomicAdd(&h[solveKey(P, i)], 1u);
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < nk; b += blockDim.x)
        if (h[b]) atomicAdd(P.lenCount + b, h[b]);
}
// exclusive prefix of the key counts into the cursors (one small block)
__global__ void __launch_bounds__(32) ptLenPrefixKernel(const PtParams P) {
    if (threadIdx.x != 0) return;
    const uint32_t nk = (P.maxBounces + 1) * kSortTypes;
    uint32_t run = 0;
    for (uint32_t b = 0; b < nk; ++b) {
        P.lenCursor[b] = run;
        run += P.lenCount[b];
    }
}
__global__ void __launch_bounds__(256) ptLenScatterKernel(const PtParams P, uint32_t* __restrict__ order) {
    __shared__ uint32_t h[kMaxKeys], base[kMaxKeys];
    const uint32_t nk = (P.maxBounces + 1) * kSortTypes;
    const uint32_t per = (P.nWave + gridDim.x - 1) / gridDim.x;
    const uint32_t begin = min(blockIdx.x * per, P.nWave), end = min(begin + per, P.nWave);
    for (uint32_t b = threadIdx.x; b < nk; b += blockDim.x) h[b] = 0;
    __syncthreads();
    for (uint32_t i = begin + threadIdx.x; i < end; i += blockDim.x) atomicAdd(&h[solveKey(P, i)], 1u);
    __syncthreads();
    // each key's cursor starts at the key's first slot (ptLenPrefixKernel)
    for (uint32_t b = threadIdx.x; b < nk; b += blockDim.x) {
        base[b] = h[b] ? atomicAdd(P.lenCursor + b, h[b]) : 0u;
        h[b] = 0;
    }
    __syncthreads();
    for (uint32_t i = begin + threadIdx.x; i < end; i += blockDim.x) {
        const uint32_t b = solveKey(P, i);
        order[base[b] + atomicAdd(&h[b], 1u)] = i;
    }
}

// The frame index word: set before the first frame, advanced after every frame.
__global__ void ptFrameKernel(uint32_t* frameDev, uint32_t frame, int advance) { *frameDev = advance ? *frameDev + 1u : frame; }

}  // namespace pltdev

namespace plt {

cudaError_t launchSetFrame(uint32_t* frameDev, uint32_t frame, bool advance, cudaStream_t stream) {
    pltdev::ptFrameKernel<<<1, 1, 0, stream>>>(frameDev, frame, advance ? 1 : 0);
    return cudaGetLastError();
}

cudaError_t launchResolve(const PtParams& p, uint32_t frames, int numSMs, cudaStream_t stream) {
    if (p.nTotal == 0) return cudaSuccess;
    const uint32_t grid = std::min<uint32_t>((p.nTotal + 255) / 256, (uint32_t)numSMs * 8);
    pltdev::ptResolveKernel<<<grid, 256, 0, stream>>>(p, 1.0 / (double)frames);
    return cudaGetLastError();
}

}  // namespace plt
