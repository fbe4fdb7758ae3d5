// One BSDF query on the device: input gather, IMaterialInstance wrappers (frame rotations,
// coherence transform), dispatch by material type, output scatter.  Paths cited are inside
// ssteinberg/PLTFalcor.
#pragma once

#include "plt_device_bsdf.cuh"
#include "plt_internal.h"

namespace pltdev {

using plt::BatchParams;

// Loads of the query planes.  A material type's queries are spread over their tile, so each
// 32-byte sector of a plane is read by several types' warps at different times.  PLT_PLANE_LOAD 1
// asks L2 to fetch the whole 128-byte line on a miss, so the neighbouring queries' reads hit L2:
// on the 2^22 mixed batch the shade kernel moves 0.80 GB instead of 0.93 GB in the same time.  2
// also skips L1 allocation: 1.58 GB and 9 % slower (warps re-read their sectors).
#ifndef PLT_PLANE_LOAD
#define PLT_PLANE_LOAD 1
#endif
PLT_DI float ldPlane(const float* p) {
#if PLT_PLANE_LOAD == 1
    float v;
    asm("ld.global.nc.L2::128B.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
#elif PLT_PLANE_LOAD == 2
    float v;
    asm("ld.global.nc.L1::no_allocate.L2::128B.f32 %0, [%1];" : "=f"(v) : "l"(p));
    return v;
#else
    return __ldg(p);
#endif
}
PLT_DI uint32_t ldPlane(const uint32_t* p) {
#if PLT_PLANE_LOAD == 1
    uint32_t v;
    asm("ld.global.nc.L2::128B.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
#elif PLT_PLANE_LOAD == 2
    uint32_t v;
    asm("ld.global.nc.L1::no_allocate.L2::128B.u32 %0, [%1];" : "=r"(v) : "l"(p));
    return v;
#else
    return __ldg(p);
#endif
}
PLT_DI f3 ld3(const float* __restrict__ p, uint32_t i, uint32_t n) { return mk3(ldPlane(p + i), ldPlane(p + n + i), ldPlane(p + 2 * n + i)); }
PLT_DI void st3(float* p, uint32_t i, uint32_t n, f3 v) { p[i] = v.x; p[n + i] = v.y; p[2 * n + i] = v.z; }

// grating frame: T = (gx, gy, 0), B = cross(N, T) = (-gy, gx, 0), N = +z
// (DiffractionGrating.slang:83-90)
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
__device__ __forceinline__ void processQueryTyped(const BatchParams& P, const Ctx& c, uint32_t i, uint32_t opMask, uint32_t mid,
                                                  uint32_t type) {
    const uint32_t n = P.q.n;
    const uint32_t ops = P.ops & opMask;
    const bool badId = mid >= P.nMats;
    const DevMaterial* __restrict__ m = P.mats + (badId ? 0u : mid);
    const f3 V = ld3(P.q.v, i, n);
    const f3 W = ld3(P.q.w, i, n);
    const uint32_t lobe = P.q.lobe ? ldPlane(P.q.lobe + i) : kLobeAll;

    DBeam<H> b;
#pragma unroll
    for (int c4 = 0; c4 < 4; ++c4)
#pragma unroll
        for (int j = 0; j < H; ++j) b.L[c4][j] = ldPlane(P.q.stokes + (size_t)(c4 * H + j) * n + i);
#pragma unroll
    for (int j = 0; j < H; ++j) b.wl[j] = ldPlane(P.q.wavelengths + (size_t)j * n + i);
    b.D0 = ldPlane(P.q.coherence + i);
    b.D1 = ldPlane(P.q.coherence + n + i);
    b.D2 = ldPlane(P.q.coherence + 2 * n + i);
    b.r_m = ldPlane(P.q.coherence + 3 * n + i);
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

// PLT_TYPE_MAJOR=1 switches on the material type once, so each case holds that material's whole
// eval + pdf + lambdaPdf + sample path (the per-op dispatches fold to one branch) and a warp's
// instruction stream stays in one region.  It measured slower on the mixed batch (4.51 against
// 4.80 G queries/s: the per-type copies of the query loads and stores grow the code by a quarter),
// so the default keeps one switch per operation.
#ifndef PLT_TYPE_MAJOR
#define PLT_TYPE_MAJOR 0
#endif
template <int H>
__device__ __forceinline__ void processQuery(const BatchParams& P, const Ctx& c, uint32_t i, uint32_t opMask = 0xFFFFFFFFu) {
    const uint32_t mid = __ldg(P.q.material + i);
    const uint32_t type = mid >= P.nMats ? 0u : __ldg(&P.mats[mid].type);
#if PLT_TYPE_MAJOR
    switch (type) {
    case kMatDielectric: processQueryTyped<H>(P, c, i, opMask, mid, kMatDielectric); break;
    case kMatConductor: processQueryTyped<H>(P, c, i, opMask, mid, kMatConductor); break;
    case kMatOpaqueDielectric: processQueryTyped<H>(P, c, i, opMask, mid, kMatOpaqueDielectric); break;
    case kMatCoatedConductor: processQueryTyped<H>(P, c, i, opMask, mid, kMatCoatedConductor); break;
    case kMatCoatedOpaque: processQueryTyped<H>(P, c, i, opMask, mid, kMatCoatedOpaque); break;
    case kMatGratedConductor: processQueryTyped<H>(P, c, i, opMask, mid, kMatGratedConductor); break;
    case kMatGratedOpaque: processQueryTyped<H>(P, c, i, opMask, mid, kMatGratedOpaque); break;
    case kMatThin: processQueryTyped<H>(P, c, i, opMask, mid, kMatThin); break;
    case kMatMultilayer: processQueryTyped<H>(P, c, i, opMask, mid, kMatMultilayer); break;
    case kMatDiffuse: processQueryTyped<H>(P, c, i, opMask, mid, kMatDiffuse); break;
    default: processQueryTyped<H>(P, c, i, opMask, mid, type); break;
    }
#else
    processQueryTyped<H>(P, c, i, opMask, mid, type);
#endif
}

}  // namespace pltdev
