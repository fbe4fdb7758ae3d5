// Fused batched BSDF kernel: one launch serves eval / pdf / sample / lambdaPdf for queries of
// any mix of PLT materials (the batched form of IMaterialInstance,
// Source/Falcor/Rendering/Materials/IMaterialInstance.slang:122-184 in ssteinberg/PLTFalcor).
//
// Work layout (sm_103a): a persistent grid walks tiles of 2048 queries.  Each CTA sorts its tile
// by material type in shared memory (counting sort: shared-atomic ranks + a 16-bin scan), so a
// warp processes one material's code path; the spectral tables (conductor IOR profiles) are
// staged into shared memory once per CTA by a bulk asynchronous copy on an mbarrier.  Inputs are
// SoA planes read through the read-only path; each tile's planes stay L1/L2-resident while its
// warps gather them, so DRAM traffic stays at one read of the inputs and one write of the
// outputs.
#include "plt_device_bsdf.cuh"
#include "plt_internal.h"
#include "plt_ptx.cuh"

namespace pltdev {

using plt::BatchParams;

PLT_DI f3 ld3(const float* __restrict__ p, uint32_t i, uint32_t n) { return mk3(__ldg(p + i), __ldg(p + n + i), __ldg(p + 2 * n + i)); }
PLT_DI void st3(float* p, uint32_t i, uint32_t n, f3 v) { p[i] = v.x; p[n + i] = v.y; p[2 * n + i] = v.z; }

// grating frame: T = (gx, gy, 0), B = cross(N, T) = (-gy, gx, 0), N = +z
struct GFrame {
    float gx, gy;
    PLT_DI f3 toLocal(f3 v) const { return mk3(v.x * gx + v.y * gy + v.z * 0.f, v.x * -gy + v.y * gx + v.z * 0.f, v.z); }
    PLT_DI f3 fromLocal(f3 v) const { return mk3(gx * v.x + -gy * v.y, gy * v.x + gx * v.y, v.z); }
};

template <int H>
PLT_DI void evalDispatch(uint32_t type, const DevMaterial* __restrict__ m, const Ctx& c, f3 V, f3 W, uint32_t lobe, DBeam<H>& b) {
    // IMaterialInstance.eval wrapper: rotate the beam to the exit frame, evaluate, transform
    // the coherence (e.g. PLTDielectricBSDF.slang:285-301).
    if (type == kMatGratedConductor || type == kMatGratedOpaque) {
        const GFrame g{__ldg(m->p + PD_GX), __ldg(m->p + PD_GY)};
        b.r = g.toLocal(b.r);
        b.t = g.toLocal(b.t);
        const f3 wi = g.toLocal(V), wo = g.toLocal(W);
        b.constructLocalFrame(wo);
        if (type == kMatGratedConductor) gratEval<H, true>(m, c, wi, wo, lobe, b);
        else gratEval<H, false>(m, c, wi, wo, lobe, b);
        int lx, ly;
        decodeGratingLobe(lobe, lx, ly);
        if (lx == 0 && ly == 0) scatterCoherence(b, wo, (lobe & kLobeDelta) != 0);
        b.r = g.fromLocal(b.r);
        b.t = g.fromLocal(b.t);
        return;
    }
    b.constructLocalFrame(W);
    switch (type) {
    case kMatDielectric: dielEval<H>(m, V, W, lobe, b); scatterCoherence(b, W, (lobe & kLobeDelta) != 0); break;
    case kMatConductor: condEval<H>(m, c, V, W, lobe, b); scatterCoherence(b, W, (lobe & kLobeDelta) != 0); break;
    case kMatOpaqueDielectric: opaqEval<H>(m, V, W, lobe, b); scatterCoherence(b, W, (lobe & kLobeDelta) != 0); break;
    case kMatCoatedConductor: coatEval<H, true>(m, c, V, W, lobe, b); scatterCoherence(b, W, (lobe & kLobeDelta) != 0); break;
    case kMatCoatedOpaque: coatEval<H, false>(m, c, V, W, lobe, b); scatterCoherence(b, W, (lobe & kLobeDelta) != 0); break;
    case kMatThin: thinEval<H>(m, V, W, lobe, b); break;
    case kMatMultilayer: mlEval<H>(m, c, V, W, lobe, b); break;
    case kMatDiffuse: diffEval<H>(m, V, lobe, b); scatterCoherence(b, W, false); break;
    default: b.setZero(); break;
    }
}

// pdf(sd, toLight = W) = bxdf.pdf(toLocal(W), toLocal(V), hero wavelength)
PLT_DI float pdfDispatch(uint32_t type, const DevMaterial* __restrict__ m, f3 V, f3 W, float wl) {
    switch (type) {
    case kMatDielectric: return dielPdf(m, W, V, wl);
    case kMatConductor: return condPdf(m, W, V, wl);
    case kMatOpaqueDielectric: return opaqPdf(m, W, V);
    case kMatCoatedConductor:
    case kMatCoatedOpaque: return coatPdf(m, W, V, wl);
    case kMatGratedConductor:
    case kMatGratedOpaque: {
        const GFrame g{__ldg(m->p + PD_GX), __ldg(m->p + PD_GY)};
        return type == kMatGratedConductor ? gratPdf<true>(m, g.toLocal(W), g.toLocal(V), wl) : gratPdf<false>(m, g.toLocal(W), g.toLocal(V), wl);
    }
    case kMatDiffuse: return V.z * k1_Pi;
    default: return 0.f;  // thin dielectric, multilayer: no non-delta lobes
    }
}

// sample(sd, sg, hero wavelength) with lobe mask All and no hint
PLT_DI bool sampleDispatch(uint32_t type, const DevMaterial* __restrict__ m, f3 V, f3& wo, float& pdf, float& weight, uint32_t& lobe,
                           SampleGen& sg, float wl) {
    switch (type) {
    case kMatDielectric: return dielSample(m, V, wo, pdf, weight, lobe, sg, wl);
    case kMatConductor: return condSample(m, V, wo, pdf, weight, lobe, sg, wl);
    case kMatOpaqueDielectric: return opaqSample(m, V, wo, pdf, weight, lobe, sg, wl);
    case kMatCoatedConductor:
    case kMatCoatedOpaque: return coatSample(m, V, wo, pdf, weight, lobe, sg, wl);
    case kMatGratedConductor:
    case kMatGratedOpaque: {
        const GFrame g{__ldg(m->p + PD_GX), __ldg(m->p + PD_GY)};
        const bool ok = type == kMatGratedConductor ? gratSample<true>(m, g.toLocal(V), wo, pdf, weight, lobe, sg, wl)
                                                    : gratSample<false>(m, g.toLocal(V), wo, pdf, weight, lobe, sg, wl);
        if (ok) wo = g.fromLocal(wo);
        return ok;
    }
    case kMatThin: return thinSample(m, V, wo, pdf, weight, lobe, sg);
    case kMatMultilayer:
        if (V.z <= 0.f) return false;
        pdf = 1.f;
        wo = reflectL(V);
        lobe = kLobeDeltaR;
        weight = m00Of(m->m00a, wl);
        return V.z * wo.z > 0.f;
    case kMatDiffuse: return diffSample(m, wo, pdf, weight, lobe, sg, wl);
    default: return false;
    }
}

template <int H>
PLT_DI void lambdaPdfDispatch(uint32_t type, const DevMaterial* __restrict__ m, f3 V, f3 W, uint32_t lobe, const DBeam<H>& b, float* out) {
    switch (type) {
    case kMatDielectric: dielLambdaPdf<H>(m, V, W, lobe, b, out); return;
    case kMatConductor:
#pragma unroll
        for (int j = 0; j < H; ++j) out[j] = (lobe & kLobeNonDelta) ? fracPdf(m->p, W, V, kOfWl(b.wl[j])) : 1.f;
        return;
    case kMatCoatedConductor:
    case kMatCoatedOpaque: coatLambdaPdf<H>(m, V, W, lobe, b, out); return;
    case kMatGratedConductor:
    case kMatGratedOpaque: gratLambdaPdf<H>(m, V, W, lobe, b, out); return;
    default:
#pragma unroll
        for (int j = 0; j < H; ++j) out[j] = 1.f;
        return;
    }
}

template <int H>
__device__ void processQuery(const BatchParams& P, const Ctx& c, uint32_t i) {
    const uint32_t n = P.q.n;
    const uint32_t mid = __ldg(P.q.material + i);
    const uint32_t ops = P.ops;
    const bool badId = mid >= P.nMats;
    const DevMaterial* __restrict__ m = P.mats + (badId ? 0u : mid);
    const uint32_t type = badId ? 0u : __ldg(&m->type);
    const f3 V = ld3(P.q.v, i, n);
    const f3 W = ld3(P.q.w, i, n);
    const uint32_t lobe = P.q.lobe ? __ldg(P.q.lobe + i) : kLobeAll;

    DBeam<H> b;
#pragma unroll
    for (int c4 = 0; c4 < 4; ++c4)
#pragma unroll
        for (int j = 0; j < H; ++j) b.L[c4][j] = __ldg(P.q.stokes + (size_t)(c4 * H + j) * n + i);
#pragma unroll
    for (int j = 0; j < H; ++j) b.wl[j] = __ldg(P.q.wavelengths + (size_t)j * n + i);
    b.D0 = __ldg(P.q.coherence + i);
    b.D1 = __ldg(P.q.coherence + n + i);
    b.D2 = __ldg(P.q.coherence + 2 * n + i);
    b.r_m = __ldg(P.q.coherence + 3 * n + i);
    b.r = -V;
    b.t = P.q.beam_t ? ld3(P.q.beam_t, i, n) : canonical_tangent(b.r);

    uint32_t st = 0;
    if (badId) st |= plt::kStatusBadMaterialId;
    else if (type == 0u || type == 1u || type >= kMatTypeCount) st |= plt::kStatusUnknownType;
    if (!(isfinite(V.x) && isfinite(V.y) && isfinite(V.z) && isfinite(W.x) && isfinite(W.y) && isfinite(W.z) && isfinite(b.wl[0])))
        st |= plt::kStatusNanInput;
    const bool ok = (st & (plt::kStatusBadMaterialId | plt::kStatusUnknownType)) == 0;

    if (ops & PLT_OP_EVAL) {
        DBeam<H> e = b;
        if (ok) evalDispatch<H>(type, m, c, V, W, lobe, e);
        else e.setZero();
        if (P.r.stokes) {
#pragma unroll
            for (int c4 = 0; c4 < 4; ++c4)
#pragma unroll
                for (int j = 0; j < H; ++j) P.r.stokes[(size_t)(c4 * H + j) * n + i] = e.L[c4][j];
        }
        if (P.r.coherence) {
            P.r.coherence[i] = e.D0;
            P.r.coherence[n + i] = e.D1;
            P.r.coherence[2 * n + i] = e.D2;
            P.r.coherence[3 * n + i] = e.r_m;
        }
        if (P.r.beam_t) st3(P.r.beam_t, i, n, e.t);
    }
    if ((ops & PLT_OP_PDF) && P.r.pdf) P.r.pdf[i] = ok ? pdfDispatch(type, m, V, W, b.wl[0]) : 0.f;
    if ((ops & PLT_OP_LAMBDA_PDF) && P.r.lambda_pdf) {
        float lp[H];
        if (ok) lambdaPdfDispatch<H>(type, m, V, W, lobe, b, lp);
        else {
#pragma unroll
            for (int j = 0; j < H; ++j) lp[j] = 0.f;
        }
#pragma unroll
        for (int j = 0; j < H; ++j) P.r.lambda_pdf[(size_t)j * n + i] = lp[j];
    }
    if (ops & PLT_OP_SAMPLE) {
        SampleGen sg;
        const uint32_t jj = i + P.q.rng_offset;
        sg.init(jj & 0xFFFFu, jj >> 16, P.q.frame);
        f3 wo = mk3(0.f, 0.f, 0.f);
        float pdf = 0.f, weight = 0.f;
        uint32_t sl = 0;
        const bool valid = ok && sampleDispatch(type, m, V, wo, pdf, weight, sl, sg, b.wl[0]);
        if (P.r.sample_wo) st3(P.r.sample_wo, i, n, wo);
        if (P.r.sample_pdf) P.r.sample_pdf[i] = pdf;
        if (P.r.sample_weight) P.r.sample_weight[i] = weight;
        if (P.r.sample_lobe) P.r.sample_lobe[i] = sl;
        if (P.r.sample_valid) P.r.sample_valid[i] = valid ? 1u : 0u;
    }
    if (st) atomicOr(P.status, st);
}

template <int H>
__global__ void __launch_bounds__(plt::kBatchThreads, 2) bsdfBatchKernel(const BatchParams P) {
    using namespace plt;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint32_t counts[16];
    __shared__ uint32_t offs[16];
    __shared__ __align__(8) uint64_t bar;

    DevProfile* sprof = reinterpret_cast<DevProfile*>(smem);
    uint16_t* perm = reinterpret_cast<uint16_t*>(smem + (size_t)P.nProfiles * sizeof(DevProfile));
    const uint32_t tid = threadIdx.x;

    // Stage the spectral profiles into shared memory with one bulk asynchronous copy.
    const uint32_t profBytes = P.nProfiles * (uint32_t)sizeof(DevProfile);
    if (profBytes > 0) {
        if (tid == 0) {
            mbar_init(&bar, 1);
            fence_mbar_init();
        }
        __syncthreads();
        if (tid == 0) {
            mbar_arrive_expect_tx(&bar, profBytes);
            bulk_g2s(sprof, P.profiles, profBytes, &bar);
        }
        const bool landed = mbar_wait_bounded(&bar, 0, 1u << 22);
        // every thread agrees before anyone leaves, so no barrier below waits on an exited thread
        if (!__syncthreads_and(landed)) {
            if (tid == 0) {
                atomicOr(P.status, kStatusCopyTimeout);
                mbar_wait_bounded(&bar, 0, 1u << 22);  // let a late copy land before the CTA leaves
            }
            return;
        }
    }
    const Ctx c{sprof, P.nProfiles, P.flags};

    const uint32_t n = P.q.n;
    const uint32_t nTiles = (n + kBatchTile - 1) / kBatchTile;
    for (uint32_t tile = blockIdx.x; tile < nTiles; tile += gridDim.x) {
        const uint32_t base = tile * kBatchTile;
        if (tid < 16) counts[tid] = 0;
        __syncthreads();
        uint8_t typ[kBatchItems];
        uint16_t rank[kBatchItems];
#pragma unroll
        for (int k = 0; k < kBatchItems; ++k) {
            const uint32_t idx = base + k * kBatchThreads + tid;
            uint32_t t = 15;
            if (idx < n) {
                const uint32_t mid = __ldg(P.q.material + idx);
                t = mid < P.nMats ? __ldg(P.matType + mid) : 14u;
            }
            typ[k] = (uint8_t)t;
            rank[k] = (uint16_t)atomicAdd(&counts[t], 1u);
        }
        __syncthreads();
        if (tid == 0) {
            uint32_t acc = 0;
#pragma unroll
            for (int t = 0; t < 16; ++t) { offs[t] = acc; acc += counts[t]; }
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kBatchItems; ++k) perm[offs[typ[k]] + rank[k]] = (uint16_t)(k * kBatchThreads + tid);
        __syncthreads();
#pragma unroll 1
        for (int k = 0; k < kBatchItems; ++k) {
            const uint32_t local = perm[k * kBatchThreads + tid];
            const uint32_t idx = base + local;
            if (idx < n) processQuery<H>(P, c, idx);
        }
        __syncthreads();
    }
}

}  // namespace pltdev

namespace plt {

// Persistent grid: SM count x resident CTAs per SM (occupancy at this launch's shared memory),
// capped by the tile count.
template <int H>
cudaError_t launchBsdfBatchH(const BatchParams& p, int numSMs, cudaStream_t stream) {
    const size_t smem = (size_t)p.nProfiles * sizeof(pltdev::DevProfile) + (size_t)kBatchTile * sizeof(uint16_t);
    static size_t cachedSmem = (size_t)-1;
    static int blocksPerSM = 1;
    if (smem != cachedSmem) {
        cudaError_t e = cudaFuncSetAttribute(pltdev::bsdfBatchKernel<H>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, pltdev::bsdfBatchKernel<H>, kBatchThreads, smem) != cudaSuccess || b < 1) b = 1;
        blocksPerSM = b;
        cachedSmem = smem;
    }
    const uint32_t nTiles = (p.q.n + kBatchTile - 1) / kBatchTile;
    uint32_t grid = (uint32_t)(numSMs * blocksPerSM);
    if (grid > nTiles) grid = nTiles;
    if (grid == 0) return cudaSuccess;
    pltdev::bsdfBatchKernel<H><<<grid, kBatchThreads, smem, stream>>>(p);
    return cudaGetLastError();
}

}  // namespace plt
