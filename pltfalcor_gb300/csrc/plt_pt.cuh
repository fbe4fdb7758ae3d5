// PLTPT render pass on the GPU: the sample pass (backward path construction,
// RenderPasses/PLTPT/pltpt_sample.rt.slang) as a wavefront of one kernel per path segment over a
// compacted queue of live paths, and the solve pass (NEE, emissive hits, forward beam replay,
// spectral MIS, measurement, pltpt_solve.rt.slang) as one thread per path.  Paths cited are inside
// ssteinberg/PLTFalcor.  The scene has identity instance transforms and untextured materials; the
// light types are emissive triangles only (no environment map, no analytic lights), so light-type
// selection (LightSampling.slangh:40-90) always picks emissive geometry after one draw.
#pragma once

// The render kernels call the large shared helpers (Fresnel, surface models, BesselJ, grating
// lobes, spectra) instead of inlining them: their divergent warps are bound by instruction fetch,
// and the smaller code measured 10-12 % faster per frame.  (The BSDF batch keeps them inlined.)
#ifndef PLT_OUTLINE_HELPERS
#define PLT_OUTLINE_HELPERS 1
#endif

#include <cuda_fp16.h>

#include "plt_bsdf_query.cuh"
#include "plt_envmap.cuh"
#include "plt_mlp.cuh"
#include "plt_bounds.cuh"
#include "plt_nvtx.h"
#include "plt_trace.cuh"

namespace pltdev {

// The render pass's material dispatchers (eval, pdf, lambdaPdf over all PLT types): PLT_PT_OUTLINE=1
// emits each once per kernel and calls it, which keeps the divergent solve kernel's code footprint
// (instruction-fetch stalls) small.
#ifndef PLT_PT_OUTLINE
#define PLT_PT_OUTLINE 0
#endif
#if PLT_PT_OUTLINE
#define PLT_PTD static __device__ __noinline__
#else
#define PLT_PTD __device__ __forceinline__
#endif

using plt::PtParams;
using plt::PtScene;

constexpr uint32_t kNoHit = 0xFFFFFFFFu;
// RayFlags, Path.slang:46-106
constexpr uint32_t kFlagLastDelta = 0x1u, kFlagDispersive = 0x2u, kFlagOnlyDelta = 0x4u, kFlagMiss = 0x10u, kFlagTerminated = 0x20u;
// a vertex where the learned proposal was a sampling technique
constexpr uint32_t kFlagLearned = 0x40u;
constexpr float kQcutoffForMS = .15f;
constexpr float kFltMax = 3.402823466e+38f;
constexpr float kFltMin = 1.175494351e-38f;

PLT_DI f3 ld3s(const float* p, uint32_t i) { return mk3(__ldg(p + 3 * i), __ldg(p + 3 * i + 1), __ldg(p + 3 * i + 2)); }
PLT_DI f3 ldPlane3(const float* p, uint32_t i, uint32_t n) { return mk3(p[i], p[n + i], p[2 * n + i]); }
PLT_DI void stPlane3(float* p, uint32_t i, uint32_t n, f3 v) { p[i] = v.x; p[n + i] = v.y; p[2 * n + i] = v.z; }
PLT_DI f3 rnormalize(f3 a) { return a / __fsqrt_rn(dot(a, a)); }
PLT_DI float hsign(float x) { return x > 0.f ? 1.f : (x < 0.f ? -1.f : 0.f); }

// ---- geometry helpers -----------------------------------------------------------------------
// computeRayOrigin, Utils/Geometry/GeometryHelpers.slang:47-60
PLT_DI float rayOriginC(float p, float n) {
    const float origin = 1.f / 16.f, fScale = 3.f / 65536.f, iScale = 3 * 256.f;
    const int iOff = (int)(n * iScale);
    const float iPos = __int_as_float(__float_as_int(p) + (p < 0.f ? -iOff : iOff));
    const float fOff = n * fScale;
    return fabsf(p) < origin ? p + fOff : iPos;
}
PLT_DI f3 computeRayOrigin(f3 p, f3 n) { return mk3(rayOriginC(p.x, n.x), rayOriginC(p.y, n.y), rayOriginC(p.z, n.z)); }

// ndir_to_oct_equal_area_snorm / oct_to_ndir_equal_area_snorm, Utils/Math/MathHelpers.slang:199-243
PLT_DI f2 ndirToOctEqualArea(f3 n) {
    const float r = sqrtf(1.f - fabsf(n.z));
    const float phi = atan2f(fabsf(n.y), fabsf(n.x));
    float py = r * phi * 0.636619772367581343076f;
    float px = r - py;
    if (n.z < 0.f) {
        const float tx = 1.f - py, ty = 1.f - px;
        px = tx;
        py = ty;
    }
    return f2{px * hsign(n.x), py * hsign(n.y)};
}
PLT_DI f3 octToNdirEqualArea(f2 p) {
    const float d = 1.f - (fabsf(p.x) + fabsf(p.y));
    const float r = 1.f - fabsf(d);
    const float phi = (r > 0.f) ? ((fabsf(p.y) - fabsf(p.x)) / r + 1.f) * 0.785398163397448309616f : 0.f;
    const float f = r * sqrtf(2.f - r * r);
    float s, c;
    sincosf(phi, &s, &c);
    return mk3(f * hsign(p.x) * c, f * hsign(p.y) * s, hsign(d) * (1.f - r * r));
}

// ---- vertex and shading data ----------------------------------------------------------------
struct VData {
    f3 posW, normalW, faceN;
    float tw[4];
};
// computeVertexData, Scene/Scene.slang:530-567 (identity world matrix)
PLT_DI VData vertexData(const PtParams& P, uint32_t prim, float b1, float b2) {
    prim = (uint32_t)pltIdx(P.status, prim, P.nTris, kSitePrim);
    const float w0 = 1.f - b1 - b2;
    const uint32_t i0 = __ldg(P.idx + 3 * prim), i1 = __ldg(P.idx + 3 * prim + 1), i2 = __ldg(P.idx + 3 * prim + 2);
    const f3 p0 = ld3s(P.pos, i0), p1 = ld3s(P.pos, i1), p2 = ld3s(P.pos, i2);
    VData v;
    v.posW = p0 * w0 + p1 * b1 + p2 * b2;
    v.normalW = rnormalize(ld3s(P.nrm, i0) * w0 + ld3s(P.nrm, i1) * b1 + ld3s(P.nrm, i2) * b2);
    v.faceN = rnormalize(cross(p1 - p0, p2 - p0));
    if (P.tan) {
        float t[4];
#pragma unroll
        for (int c = 0; c < 4; ++c) t[c] = __ldg(P.tan + 4 * i0 + c) * w0 + __ldg(P.tan + 4 * i1 + c) * b1 + __ldg(P.tan + 4 * i2 + c) * b2;
        const f3 tx = rnormalize(mk3(t[0], t[1], t[2]));
        v.tw[0] = tx.x; v.tw[1] = tx.y; v.tw[2] = tx.z; v.tw[3] = hsign(t[3]);
    } else {
        v.tw[0] = v.tw[1] = v.tw[2] = v.tw[3] = 0.f;
    }
    return v;
}

struct SD {
    f3 posW, V, N, T, B, faceN;
    bool frontFacing;
    PLT_DI f3 toLocal(f3 v) const { return mk3(dot(v, T), dot(v, B), dot(v, N)); }
    PLT_DI f3 fromLocal(f3 v) const { return T * v.x + B * v.y + N * v.z; }
    // ShadingData.computeNewRayOrigin, Scene/ShadingData.slang:77-80
    PLT_DI f3 newRayOrigin(bool viewside) const { return computeRayOrigin(posW, (frontFacing == viewside) ? faceN : -faceN); }
};
// computeNewRayOrigin(sd, dir), ShadowRays.slangh:50-52
PLT_DI f3 newRayOriginToward(const SD& sd, f3 dir) { return computeRayOrigin(sd.posW, dot(sd.faceN, dir) >= 0.f ? sd.faceN : -sd.faceN); }

// prepareShadingData, Scene/Material/MaterialFactory.slang:79-128 with computeTangentSpace
// (Scene/Material/ShadingUtils.slang:126-153,243-251); double-sided materials flip N on back faces.
PLT_DI SD prepareSD(const VData& v, uint32_t props, f3 viewDir) {
    SD sd;
    sd.posW = v.posW;
    sd.V = viewDir;
    sd.N = v.normalW;
    const f3 t = mk3(v.tw[0], v.tw[1], v.tw[2]);
    const float NdotT = dot(t, sd.N);
    const bool valid = fabsf(v.tw[3]) == 1.0f && dot(t, t) > 0.f && fabsf(NdotT) < 0.9999f;
    if (valid) {
        sd.T = rnormalize(t - sd.N * NdotT);
        sd.B = cross(sd.N, sd.T) * v.tw[3];
    } else {
        sd.T = perp_stark(sd.N);
        sd.B = cross(sd.N, sd.T);
    }
    sd.faceN = v.faceN;
    sd.frontFacing = dot(sd.V, sd.faceN) >= 0.f;
    if (!sd.frontFacing && (props & plt::kPropDoubleSided)) sd.N = -sd.N;
    return sd;
}

// ---- material instance in world space (IMaterialInstance wrappers of PLT*BSDF.slang) ----------
struct WFrame {
    f3 T, B, N;
    PLT_DI f3 toLocal(f3 v) const { return mk3(dot(v, T), dot(v, B), dot(v, N)); }
    PLT_DI f3 fromLocal(f3 v) const { return T * v.x + B * v.y + N * v.z; }
};
PLT_DI bool isGrated(uint32_t type) { return type == kMatGratedConductor || type == kMatGratedOpaque; }
// sd frame, or localGratingShadingFrame (DiffractionGrating.slang:83-90) for the grated materials
PLT_DI WFrame bsdfFrame(const SD& sd, uint32_t type, const DevMaterial* __restrict__ m) {
    WFrame f;
    if (isGrated(type)) {
        f.T = sd.fromLocal(mk3(__ldg(m->p + PD_GX), __ldg(m->p + PD_GY), 0.f));
        f.N = sd.N;
        f.B = cross(f.N, f.T);
    } else {
        f.T = sd.T;
        f.B = sd.B;
        f.N = sd.N;
    }
    return f;
}

template <int H>
PLT_PTD void ptEval(const DevMaterial* __restrict__ m, uint32_t type, const Ctx& c, const SD& sd, f3 toEye, uint32_t lobe, DBeam<H>& b) {
    const WFrame F = bsdfFrame(sd, type, m);
    b.r = F.toLocal(b.r);
    b.t = F.toLocal(b.t);
    const f3 wi = F.toLocal(sd.V), wo = F.toLocal(toEye);
    b.constructLocalFrame(wo);
    switch (type) {
    case kMatDielectric: dielEval<H>(m, wi, wo, lobe, b); scatterCoherence(b, wo, (lobe & kLobeDelta) != 0); break;
    case kMatConductor: condEval<H>(m, c, wi, wo, lobe, b); scatterCoherence(b, wo, (lobe & kLobeDelta) != 0); break;
    case kMatOpaqueDielectric: opaqEval<H>(m, wi, wo, lobe, b); scatterCoherence(b, wo, (lobe & kLobeDelta) != 0); break;
    case kMatCoatedConductor: coatEval<H, true>(m, c, wi, wo, lobe, b); scatterCoherence(b, wo, (lobe & kLobeDelta) != 0); break;
    case kMatCoatedOpaque: coatEval<H, false>(m, c, wi, wo, lobe, b); scatterCoherence(b, wo, (lobe & kLobeDelta) != 0); break;
    case kMatGratedConductor:
    case kMatGratedOpaque: {
        if (type == kMatGratedConductor) gratEval<H, true>(m, c, wi, wo, lobe, b);
        else gratEval<H, false>(m, c, wi, wo, lobe, b);
        int lx, ly;
        decodeGratingLobe(lobe, lx, ly);
        if (lx == 0 && ly == 0) scatterCoherence(b, wo, (lobe & kLobeDelta) != 0);
        break;
    }
    case kMatThin: thinEval<H>(m, wi, wo, lobe, b); break;
    case kMatMultilayer: mlEval<H>(m, c, wi, wo, lobe, b); break;
    case kMatDiffuse: diffEval<H>(m, wi, lobe, b); scatterCoherence(b, wo, false); break;
    default: b.setZero(); break;
    }
    b.r = F.fromLocal(b.r);
    b.t = F.fromLocal(b.t);
}

// sample(sd, sg, result, wavelength, lobeMask, woHint): the dielectric and thin dielectric
// restrict the lobes to the hint's side (PLTDielectricBSDF.slang:310-321,
// PLTThinDielectricBSDF.slang:230-243), the grated materials take the diffraction order closest to
// the hint; the sample pass uses lobeMask All and no hint.
// uw (x >= 0): primary sample of the surface model's direction sampler (used by the non-delta lobes)
PLT_DI bool ptSample(const DevMaterial* __restrict__ m, uint32_t type, const SD& sd, SampleGen& sg, float wl, f3& wo, float& pdf,
                     float& weight, uint32_t& lobe, uint32_t lobeMask = kLobeAll, f3 woHint = f3{0.f, 0.f, 0.f}, f2 uw = kNoWarp) {
    const WFrame F = bsdfFrame(sd, type, m);
    const f3 V = F.toLocal(sd.V);
    uint32_t sideMask = lobeMask;
    if (type == kMatDielectric || type == kMatThin) {
        const float dh = dot(sd.V, woHint);
        sideMask = (dh > 0.f ? kLobeReflection : dh < 0.f ? kLobeTransmission : kLobeAll) & lobeMask;
    }
    bool ok;
    switch (type) {
    case kMatDielectric: ok = dielSample(m, V, wo, pdf, weight, lobe, sg, wl, sideMask, uw); break;
    case kMatConductor: ok = condSample(m, V, wo, pdf, weight, lobe, sg, wl, lobeMask, uw); break;
    case kMatOpaqueDielectric: ok = opaqSample(m, V, wo, pdf, weight, lobe, sg, wl, lobeMask, uw); break;
    case kMatCoatedConductor:
    case kMatCoatedOpaque: ok = coatSample(m, V, wo, pdf, weight, lobe, sg, wl, lobeMask, uw); break;
    case kMatGratedConductor: ok = gratSample<true>(m, V, wo, pdf, weight, lobe, sg, wl, lobeMask, F.toLocal(woHint), uw); break;
    case kMatGratedOpaque: ok = gratSample<false>(m, V, wo, pdf, weight, lobe, sg, wl, lobeMask, F.toLocal(woHint), uw); break;
    case kMatThin: ok = thinSample(m, V, wo, pdf, weight, lobe, sg, sideMask); break;
    case kMatMultilayer:
        if ((lobeMask & kLobeReflection) == 0 || (lobeMask & kLobeDelta) == 0 || V.z <= 0.f) { ok = false; break; }
        pdf = 1.f;
        wo = reflectL(V);
        lobe = kLobeDeltaR;
        weight = m00Of(m->m00a, wl);
        ok = V.z * wo.z > 0.f;
        break;
    case kMatDiffuse: ok = diffSample(m, wo, pdf, weight, lobe, sg, wl) && (lobeMask & kLobeDiffuseR) != 0; break;
    default: ok = false; break;
    }
    if (ok || type == kMatDielectric) wo = F.fromLocal(wo);
    return ok;
}

PLT_PTD float ptPdf(const DevMaterial* __restrict__ m, uint32_t type, const SD& sd, f3 toLight, float wl) {
    const WFrame F = bsdfFrame(sd, type, m);
    const f3 V = F.toLocal(sd.V), W = F.toLocal(toLight);
    switch (type) {
    case kMatDielectric: return dielPdf(m, W, V, wl);
    case kMatConductor: return condPdf(m, W, V, wl);
    case kMatOpaqueDielectric: return opaqPdf(m, W, V);
    case kMatCoatedConductor:
    case kMatCoatedOpaque: return coatPdf(m, W, V, wl);
    case kMatGratedConductor: return gratPdf<true>(m, W, V, wl);
    case kMatGratedOpaque: return gratPdf<false>(m, W, V, wl);
    case kMatDiffuse: return V.z * k1_Pi;
    default: return 0.f;
    }
}

// lambdaPdf in the sd frame for every material (the grated wrappers too, PLTDiffractionGrated*BSDF)
template <int H>
PLT_PTD void ptLambdaPdf(const DevMaterial* __restrict__ m, uint32_t type, const SD& sd, f3 wo, uint32_t lobe, const DBeam<H>& bIn, float* out) {
    DBeam<H> b = bIn;
    b.r = sd.toLocal(b.r);
    b.t = sd.toLocal(b.t);
    lambdaPdfDispatch<H>(type, m, sd.toLocal(sd.V), sd.toLocal(wo), lobe, b, out);
}

// ---- spectra --------------------------------------------------------------------------------
// rgbToSpectrum of white (1, 1, 1) = the white basis (SpectrumUtils.slang:106-198)
PLT_DI float whiteSpectrum(float wl) {
    const float w[11] = {1.0000f, 1.0000f, 0.9999f, 0.9993f, 0.9992f, 0.9998f, 1.0000f, 1.0000f, 1.0000f, 1.0000f, 0.0f};
    const int b = spectrumBin(wl);
    float r = w[0];
#pragma unroll
    for (int i = 1; i < 11; ++i) r = b == i ? w[i] : r;
    return r;
}
// SpectrumSampler.hwssWavelengths, Utils/Color/SpectrumSampler.slang:43-54
template <int H> PLT_DI void hwssWavelengths(float hero, float* wl) {
    const float span = 720.0f - 380.0f;
#pragma unroll
    for (int i = 0; i < H; ++i) {
        float w = hero + float(i) * (span / float(H));
        w -= w > 720.0f ? span : 0.f;
        wl[i] = w;
    }
}
// Scene.sampleSpectrum, Scene/Scene.slang:295-330 (importance sampling draws three numbers)
template <int H>
PLT_DI void sampleSpectrum(const PtParams& P, uint32_t id, float hero, SampleGen& sg, bool importance, float* le, float* wl) {
#pragma unroll
    for (int j = 0; j < H; ++j) { le[j] = 0.f; wl[j] = 0.f; }
    if (id == kNoProfile || id >= P.nProfiles) return;
    if (importance) {
        const DevProfile& sp = P.profiles[id];
        wl[0] = hero;
        le[0] = evalSpectrum(P.profiles, P.nProfiles, id, hero);
        // the reference draws three numbers (sampleNext3D) for its at most three companion
        // wavelengths; beyond HWSS 4 one number per companion
        constexpr int kDraws = H - 1 > 3 ? H - 1 : 3;
        float x[kDraws];
#pragma unroll
        for (int c = 0; c < kDraws; ++c) x[c] = float(sp.bins) * sg.next1D();
        const float* icdf = P.profileIcdf + 128 * id;
#pragma unroll
        for (int j = 1; j < H; ++j) {
            const uint32_t i = (uint32_t)x[j - 1];
            const float a = i < sp.bins ? __ldg(icdf + i) : 1.f;
            const float b = i + 1 < sp.bins ? __ldg(icdf + i + 1) : 1.f;
            const float fr = x[j - 1] - floorf(x[j - 1]);
            const float cdf = a + (b - a) * fr;
            wl[j] = sp.minl + (sp.maxl - sp.minl) * cdf;
            le[j] = sp.intensity / (float)sp.bins;
        }
    } else {
        hwssWavelengths<H>(hero, wl);
#pragma unroll
        for (int j = 0; j < H; ++j) le[j] = evalSpectrum(P.profiles, P.nProfiles, id, wl[j]);
    }
}
PLT_DI float cieG(float x, float mu, float s1, float s2) {
    const float t = (x - mu) * (x < mu ? s1 : s2);
    return expf(-0.5f * t * t);
}
// wavelengthToD65, SpectrumUtils.slang:66-82
PLT_DI float d65(float l) {
    constexpr float t[69] = {49.9755f, 52.3118f, 54.6482f, 68.7015f, 82.7549f, 87.1204f, 91.486f, 92.4589f, 93.4318f, 90.057f,
                             86.6823f, 95.7736f, 104.865f, 110.936f, 117.008f, 117.41f, 117.812f, 116.336f, 114.861f, 115.392f,
                             115.923f, 112.367f, 108.811f, 109.082f, 109.354f, 108.578f, 107.802f, 106.296f, 104.79f, 106.239f,
                             107.689f, 106.047f, 104.405f, 104.225f, 104.046f, 102.023f, 100.f, 98.1671f, 96.3342f, 96.0611f,
                             95.788f, 92.2368f, 88.6856f, 89.3459f, 90.0062f, 89.8026f, 89.5991f, 88.6489f, 87.6987f, 85.4936f,
                             83.2886f, 83.4939f, 83.6992f, 81.863f, 80.0268f, 80.1207f, 80.2146f, 81.2462f, 82.2778f, 80.281f,
                             78.2842f, 74.0027f, 69.7213f, 70.6652f, 71.6091f, 72.979f, 74.349f, 67.9765f, 61.604f};
    const float r = (l - 380.0f) * 0.2f;
    const int hi = min(68, max(0, int(ceilf(r) + .5f))), lo = min(68, max(0, int(floorf(r) + .5f)));
    const float w = r - float(lo);
    return t[hi] * w + t[lo] * (1.0f - w);
}
// spectrumToRgb, SpectrumUtils.slang:92-104 (+ XYZtoRGB_Rec709, ColorHelpers.slang:61-70)
template <int H> PLT_DI f3 spectrumToRgb(const float* L, const float* wl, int samples) {
    float r = 0.f, g = 0.f, bl = 0.f;
#pragma unroll
    for (int i = 0; i < H; ++i) {
        if (i >= samples) break;
        const float l = wl[i];
        const float s = d65(l) * L[i];
        const float X = (0.362f * cieG(l, 442.0f, 0.0624f, 0.0374f) + 1.056f * cieG(l, 599.8f, 0.0264f, 0.0323f) -
                         0.065f * cieG(l, 501.1f, 0.0490f, 0.0382f)) * s;
        const float Y = (0.821f * cieG(l, 568.8f, 0.0213f, 0.0247f) + 0.286f * cieG(l, 530.9f, 0.0613f, 0.0322f)) * s;
        const float Z = (1.217f * cieG(l, 437.0f, 0.0845f, 0.0278f) + 0.681f * cieG(l, 459.0f, 0.0385f, 0.0725f)) * s;
        r += 3.240969941904522f * X + -1.537383177570094f * Y + -0.4986107602930032f * Z;
        g += -0.9692436362808803f * X + 1.875967501507721f * Y + 0.04155505740717569f * Z;
        bl += 0.05563007969699373f * X + -0.2039769588889765f * Y + 1.056971514242878f * Z;
    }
    const float inv = 1.f / 10.5670762f;
    return mk3(r * inv, g * inv, bl * inv);
}

// ---- beams ----------------------------------------------------------------------------------
template <int H> struct PBeam {
    DBeam<H> b;
    float spdf[H];
    f3 posW;
    int comps;
    bool distant;                 // sourced by a distant light: propagation leaves the coherence alone
};
// pltSourceBeamArea, Rendering/PLT.slang:276-290 (unpolarised, diffusivity A * I, r = 0)
template <int H>
PLT_DI void sourceBeamArea(PBeam<H>& pb, f3 posW, f3 dir, float A, float dist, const float* Le, const float* wl, float maxBeamOmega) {
    const float r2 = sqr(dist * 1e+3f);
    A = fminf(A, maxBeamOmega * r2);
#pragma unroll
    for (int j = 0; j < H; ++j) {
        pb.b.L[0][j] = Le[j];
        pb.b.L[1][j] = pb.b.L[2][j] = pb.b.L[3][j] = 0.f;
        pb.b.wl[j] = wl[j];
        pb.spdf[j] = 1.f;
    }
    pb.b.D0 = A; pb.b.D1 = 0.f; pb.b.D2 = A;
    pb.b.r_m = 0.f;
    pb.b.r = dir;
    pb.b.t = perp_stark(dir);
    pb.posW = posW;
    pb.comps = H;
    pb.distant = false;
}
// pltSourceBeamDistant, Rendering/PLT.slang:253-267: unpolarised, diffusivity min(solidAngle,
// maxOmega) I, coherence radius 1 mm, flagged distant for the beam's whole life (PLT.slang:99-114,
// 224-230)
template <int H>
PLT_DI void sourceBeamDistant(PBeam<H>& pb, f3 dir, float solidAngle, const float* Le, const float* wl, float maxBeamOmega) {
    const float omega = fminf(solidAngle, maxBeamOmega);
#pragma unroll
    for (int j = 0; j < H; ++j) {
        pb.b.L[0][j] = Le[j];
        pb.b.L[1][j] = pb.b.L[2][j] = pb.b.L[3][j] = 0.f;
        pb.b.wl[j] = wl[j];
        pb.spdf[j] = 1.f;
    }
    pb.b.D0 = omega; pb.b.D1 = 0.f; pb.b.D2 = omega;
    pb.b.r_m = 1e-3f;
    pb.b.r = dir;
    pb.b.t = perp_stark(dir);
    pb.posW = mk3(0.f, 0.f, 0.f);
    pb.comps = H;
    pb.distant = true;
}
template <int H> PLT_DI void propagate(PBeam<H>& pb, f3 p) {
    if (!pb.distant) pb.b.r_m += sqrtf(dot(p - pb.posW, p - pb.posW));
    pb.posW = p;
}
template <int H> PLT_DI void scaleBeam(PBeam<H>& pb, float s) {
#pragma unroll
    for (int c = 0; c < 4; ++c)
#pragma unroll
        for (int j = 0; j < H; ++j) pb.b.L[c][j] *= s;
}

PLT_DI float misWeight(float p0, float p1) { return p0 / (p0 + p1); }

// ---- sample pass ----------------------------------------------------------------------------
// The scene of path pid: the last scene whose first path is <= pid (scenes in path order).
PLT_DI uint32_t sceneOf(const PtParams& P, uint32_t pid) {
    uint32_t lo = 0, hi = P.nScenes;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(&P.scenes[mid].pixelBase) <= pid) lo = mid;
        else hi = mid;
    }
    return lo;
}
PLT_DI f3 camPos(const PtScene& S) { return mk3(S.cam.pos[0], S.cam.pos[1], S.cam.pos[2]); }

// Camera.computeRayPinhole, Scene/Camera/Camera.slang:46-78
PLT_DI f3 cameraDir(const PtScene& S, uint32_t px, uint32_t py) {
    float p0 = (float(px) + 0.5f) / float(S.width);
    float p1 = (float(py) + 0.5f) / float(S.height);
    p0 += -S.cam.jitter_x;
    p1 += S.cam.jitter_y;
    const float ndcx = 2.f * p0 + -1.f, ndcy = -2.f * p1 + 1.f;
    const f3 U = mk3(S.cam.u[0], S.cam.u[1], S.cam.u[2]), V = mk3(S.cam.v[0], S.cam.v[1], S.cam.v[2]);
    const f3 W = mk3(S.cam.w[0], S.cam.w[1], S.cam.w[2]);
    return rnormalize(U * ndcx + V * ndcy + W);
}

// Algorithmic traversal bytes of a thread's rays (64-byte nodes visited, 48-byte triangles
// tested), summed per warp into the frame statistics (slot 3).
PLT_DI void addTraversalBytes(const PtParams& P, uint32_t nodeVisits, uint32_t triTests) {
    unsigned long long b = 64ull * nodeVisits + 48ull * triTests;
    for (int o = 16; o > 0; o >>= 1) b += __shfl_down_sync(0xFFFFFFFFu, b, o);
    if ((threadIdx.x & 31u) == 0 && b) atomicAdd(P.stats + 3, b);
}

PLT_DI uint32_t warpAggregatedAdd(uint32_t* counter, bool pred) {
    const uint32_t mask = __ballot_sync(__activemask(), pred);
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t leader = mask ? (uint32_t)(__ffs(mask) - 1) : 0u;
    uint32_t base = 0;
    if (mask && lane == leader) base = atomicAdd(counter, (uint32_t)__popc(mask));
    base = __shfl_sync(__activemask(), base, (int)leader);
    return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

#ifdef PLT_PT_SAMPLE_PASS   // defined by plt_pt.cu only: one copy of the sample-pass kernels
__global__ void __launch_bounds__(128) ptInitKernel(const PtParams P) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < P.nWave; i += gridDim.x * blockDim.x) {
        const uint32_t gp = P.pidBase + i;
        const PtScene& S = P.scenes[sceneOf(P, gp)];
        const uint32_t local = gp - S.pixelBase;
        const uint32_t px = local % S.width, py = local / S.width;
        SampleGen sg;
        sg.init(px, py, *P.frameDev, (P.opt & plt::kPtTinySg) != 0);
        const float wl = 380.0f + sg.next1D() * (720.0f - 380.0f);   // SpectrumSampler.sampleOne
        const f3 d = cameraDir(S, px, py);
        const uint32_t n = P.npix;
        P.sg[i] = sg.s0; P.sg[n + i] = sg.s1; P.sg[2 * n + i] = sg.s2; P.sg[3 * n + i] = sg.s3;
        stPlane3(P.org, i, n, camPos(S));
        stPlane3(P.dir, i, n, d);
        P.wl[i] = wl;
        P.weight[i] = 1.f;
        P.pdf[i] = 1.f;
        P.thp[i] = 1.f;
        P.lndp[i] = 0.f;
        P.pflags[i] = kFlagOnlyDelta;
        P.plen[i] = 0;
        if (P.wpss) P.wpss[i] = 1.f;
    }
}

// One segment of every live path: TraceRay + scatterTriangleMeshClosestHit / scatterMiss
// (pltpt_sample.rt.slang:56-141), appendBounce (pltpt.slangh:138-154).  Live paths are compacted
// into the next queue with one atomic per warp.
//
// LEARNED adds the learned proposal at every proposal vertex (an enabled material hit from the
// front with wi above the shading plane).  The warp runs the network on its 32 lanes' feature rows
// (tensor cores, weights in shared memory); the network's mixture is a density q over the primary
// sample (u0, u1) in [0,1)^2 that the surface model's direction sampler turns into wo.  The primary
// sample comes from q with probability c and is uniform otherwise (one-sample MIS in primary sample
// space), so a non-delta direction has the density p(wo) * (c q(u) + 1 - c): the path weight is
// divided by that factor (kept in the path state), while the analytic pdf the reference's MIS
// weights, Russian roulette and the path-pdf cutoff use is unchanged.  The estimate therefore has
// the analytic tracer's expectation whatever the network outputs; the exact BSDF is evaluated as
// before.  A primary sample of q outside the unit square ends a path that takes a non-delta lobe.
// Residency of the analytic variant (blocks of 128 per SM; the register budget follows from it).
// The segment's closest hits, traced ahead of the segment kernel by ptSegTraceKernel.
PLT_DI TraceResult segmentHit(const PtParams& P, uint32_t slot) {
    TraceResult h;
    h.prim = P.segPrim[slot];
    h.t = 0.f;
    h.b1 = P.segBary[slot];
    h.b2 = P.segBary[P.npix + slot];
    return h;
}

// The closest hits of a segment's queue (the rays the paths continue along), traced with dynamic
// fetch (dynamicTraversal) ahead of the segment kernel, which then shades them: traversal alone
// keeps a warp's lanes full (a lane whose ray has finished takes the next one) where, inside the
// segment kernel, every lane waited for the longest ray of its warp and then for the shading of
// each other's materials.  Each CTA traces a contiguous share of the queue's slots.
// The material-type key of a segment hit for the shading order (kSegKeys - 1 for a miss).
PLT_DI uint32_t segKey(const PtParams& P, uint32_t prim) {
    if (prim >= P.nTris) return plt::kSegKeys - 1u;
    return min(__ldg(&P.mats[__ldg(P.triMat + prim)].type), plt::kSegKeys - 2u);
}

__global__ void __launch_bounds__(128) ptSegTraceKernel(const PtParams P, uint32_t it) {
    __shared__ uint32_t next, hist[plt::kSegKeys];
    const uint32_t n = P.npix;
    if (threadIdx.x < plt::kSegKeys) hist[threadIdx.x] = 0u;
    const uint32_t count = it == 0 ? P.nWave : *((volatile uint32_t*)(P.qcount + it));
    const uint32_t* qin = (it & 1u) ? P.queue0 : P.queue1;
    const uint32_t per = (count + gridDim.x - 1) / gridDim.x;
    const uint32_t begin = min(blockIdx.x * per, count), end = min(begin + per, count);
    if (threadIdx.x == 0) next = begin;
    __syncthreads();
    uint32_t nv = 0, tt = 0, overflow = 0;
    dynamicTraversal<false>(
        reinterpret_cast<const float4*>(P.nodes), P.tris, kStackDepth, end, &next,
        [&](uint32_t slot) {
            const uint32_t pid = (uint32_t)pltIdx(P.status, it == 0 ? slot : qin[pltIdx(P.status, slot, n, kSiteQueue)], n, kSitePath);
            const f3 org = ldPlane3(P.org, pid, n), dir = ldPlane3(P.dir, pid, n);
            return TravRay{org.x, org.y, org.z, dir.x, dir.y, dir.z, 0.f, kFltMax, (int32_t)__ldg(&P.scenes[sceneOf(P, P.pidBase + pid)].root)};
        },
        [&](uint32_t slot, uint32_t prim, float, float b1, float b2) {
            P.segPrim[slot] = prim;
            P.segBary[slot] = b1;
            P.segBary[n + slot] = b2;
            if (P.segOrder) atomicAdd(&hist[segKey(P, prim)], 1u);
        },
        nv, tt, overflow);
    if (overflow) atomicOr(P.status, plt::kStatusStackOverflow);
    addTraversalBytes(P, nv, tt);
    if (P.segOrder) {
        __syncthreads();
        if (threadIdx.x < plt::kSegKeys && hist[threadIdx.x]) atomicAdd(P.segSort + it * plt::kSegSortWords + threadIdx.x, hist[threadIdx.x]);
    }
}

// The segment's shading order: its queue slots counting-sorted by the hit's material type (keys
// counted by ptSegTraceKernel), so the segment kernel's warps, which take consecutive positions of
// this order from one counter, shade one material at a time and an SM's resident warps one or two.
// Each block reserves its share of each key's positions after the exclusive prefix of the counts.
__global__ void __launch_bounds__(256) ptSegScatterKernel(const PtParams P, uint32_t it) {
    __shared__ uint32_t h[plt::kSegKeys], base[plt::kSegKeys];
    const uint32_t count = it == 0 ? P.nWave : *((volatile uint32_t*)(P.qcount + it));
    const uint32_t per = (count + gridDim.x - 1) / gridDim.x;
    const uint32_t begin = min(blockIdx.x * per, count), end = min(begin + per, count);
    uint32_t* cnt = P.segSort + it * plt::kSegSortWords;
    if (threadIdx.x < plt::kSegKeys) h[threadIdx.x] = 0u;
    __syncthreads();
    for (uint32_t i = begin + threadIdx.x; i < end; i += blockDim.x) atomicAdd(&h[segKey(P, P.segPrim[i])], 1u);
    __syncthreads();
    if (threadIdx.x < plt::kSegKeys) {
        uint32_t prefix = 0;
        for (uint32_t k = 0; k < threadIdx.x; ++k) prefix += cnt[k];
        base[threadIdx.x] = h[threadIdx.x] ? prefix + atomicAdd(cnt + plt::kSegKeys + threadIdx.x, h[threadIdx.x]) : 0u;
        h[threadIdx.x] = 0u;
    }
    __syncthreads();
    for (uint32_t i = begin + threadIdx.x; i < end; i += blockDim.x) {
        const uint32_t k = segKey(P, P.segPrim[i]);
        P.segOrder[pltIdx(P.status, base[k] + atomicAdd(&h[k], 1u), count, kSiteQueue)] = i;
    }
}

#ifndef PLT_BOUNCE_MIN_BLOCKS
#define PLT_BOUNCE_MIN_BLOCKS 7
#endif
template <bool LEARNED>
__global__ void __launch_bounds__(128, LEARNED ? 3 : PLT_BOUNCE_MIN_BLOCKS) ptBounceKernel(const PtParams P, uint32_t it) {
    extern __shared__ __align__(16) unsigned char ptSmem[];
    const uint32_t n = P.npix;
    const uint32_t count = it == 0 ? P.nWave : *((volatile uint32_t*)(P.qcount + it));
    const uint32_t* qin = (it & 1u) ? P.queue0 : P.queue1;
    uint32_t* qout = (it & 1u) ? P.queue1 : P.queue0;
    const float4* nodes = reinterpret_cast<const float4*>(P.nodes);
    uint32_t nv = 0, tt = 0, overflow = 0, recorded = 0;
    const Ctx c{P.profiles, P.nProfiles, P.flags};
    (void)c;
    mlp::bf16* wbuf = nullptr;
    if constexpr (LEARNED) {
        mlp::loadNet(*reinterpret_cast<mlp::SmemNet*>(ptSmem), static_cast<const mlp::bf16*>(P.propNet));
        wbuf = reinterpret_cast<mlp::bf16*>(ptSmem + sizeof(mlp::SmemNet)) + (threadIdx.x >> 5) * 32 * mlp::kSWH;
        __syncthreads();
    }
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t rounds = (count + stride - 1) / stride;
    for (uint32_t rr = 0; rr < rounds; ++rr) {
        const uint32_t pos = rr * stride + blockIdx.x * blockDim.x + threadIdx.x;
        const bool act = pos < count;
        const uint32_t slot = act && P.segOrder ? P.segOrder[pos] : pos;   // the shading order when sorted
        bool live = false;
        uint32_t pid = 0;
        SampleGen sg;
        f3 org = mk3(0.f, 0.f, 0.f), dir = mk3(0.f, 0.f, 1.f);
        float weight = 0.f, pdf = 0.f, thp = 0.f, lndp = 0.f, wavelength = 0.f;
        float wps = 1.f;   // product of the primary-sample MIS densities (learned proposal)
        uint32_t flags = 0, len = 0;
        // the vertex this segment reaches
        bool hit = false, shouldEnd = false;
        TraceResult h;
        SD sd;
        uint32_t mid = 0;
        uint2 props = make_uint2(0u, 0u);
        float rcpThp = 1.f;
        auto append = [&](uint32_t prim, float b1, float b2, f3 wi, uint32_t lobe, uint32_t extra) {
            len = (uint32_t)pltIdx(P.status, len, (size_t)P.maxBounces + 1, kSiteBounce);
            const size_t o = (size_t)len * n + pid;
            P.bFlags[o] = flags | extra;
            P.bPrim[o] = prim;
            P.bBary[(size_t)len * 2 * n + pid] = b1;
            P.bBary[(size_t)len * 2 * n + n + pid] = b2;
            const f2 e = ndirToOctEqualArea(wi);
            P.bEw[(size_t)len * 2 * n + pid] = e.x;
            P.bEw[(size_t)len * 2 * n + n + pid] = e.y;
            P.bLobe[o] = lobe;
            P.bLndp[o] = lndp;
            P.bContrib[o] = 1.f / (pdf * thp * wps);
            ++recorded;
        };
        if (act) {
            pid = (uint32_t)pltIdx(P.status, it == 0 ? slot : qin[pltIdx(P.status, slot, n, kSiteQueue)], n, kSitePath);
            sg.s0 = P.sg[pid]; sg.s1 = P.sg[n + pid]; sg.s2 = P.sg[2 * n + pid]; sg.s3 = P.sg[3 * n + pid];
            sg.tiny = (P.opt & plt::kPtTinySg) != 0;
            org = ldPlane3(P.org, pid, n);
            dir = ldPlane3(P.dir, pid, n);
            weight = P.weight[pid]; pdf = P.pdf[pid]; thp = P.thp[pid]; lndp = P.lndp[pid];
            flags = P.pflags[pid]; len = P.plen[pid];
            wavelength = P.wl[pid];
            if constexpr (LEARNED) wps = P.wpss[pid];
            for (int guard = 0; guard < 64; ++guard) {
                if (guard == 0 && P.segPrim) h = segmentHit(P, slot);
                else
                    h = traverse<false>(nodes, P.tris, org.x, org.y, org.z, dir.x, dir.y, dir.z, 0.f, kFltMax, nv, tt, overflow,
                                        __ldg(&P.scenes[sceneOf(P, P.pidBase + pid)].root));
                const f3 wi = -dir;
                if (h.prim == kNoHit) {
                    flags |= kFlagMiss;
                    append(kNoHit, 0.f, 0.f, wi, 0u, 0u);
                    break;
                }
                const VData v = vertexData(P, h.prim, h.b1, h.b2);
                mid = (uint32_t)pltIdx(P.status, __ldg(P.triMat + h.prim), P.nMats, kSiteMaterial);
                props = __ldg(P.matProps + mid);
                sd = prepareSD(v, props.x, wi);
                if ((props.x & plt::kPropAlphaZero) && (P.opt & plt::kPtAlphaMask)) {   // alpha mask: continue the same ray
                    org = sd.newRayOrigin(false);
                    continue;
                }
                // Russian roulette RR(1 - weight, 2, u) (pltpt.slangh:170-176); pow of a negative
                // base is NaN as in the shader
                if (P.opt & plt::kPtDoRR) {
                    const float rrVal = 1.f - weight;
                    const float p = rrVal < 0.f ? __int_as_float(0x7fffffff) : rrVal * rrVal;
                    const float u = sg.next1D();
                    rcpThp = u < p ? 0.f : 1.f - p;
                }
                shouldEnd = len == P.maxBounces || (rcpThp == 0.f && len > 0);
                hit = true;
                break;
            }
            if (!hit && (flags & kFlagMiss) == 0) {
                // 64 alpha-masked hits in a row: end the path with an empty terminal record
                flags |= kFlagTerminated;
                append(kNoHit, 0.f, 0.f, -dir, 0u, 0u);
            }
        }
        // learned proposal: the warp's network inference (all 32 lanes, uniform branch)
        mlp::PropMix mix;
        bool useNet = false;
        if constexpr (LEARNED) {
            float4 mf = make_float4(0.f, 0.f, 0.f, 0.f);
            f3 wiL = mk3(0.f, 0.f, 0.f);
            if (hit) {
                mf = __ldg(P.matFeat + mid);
                wiL = sd.toLocal(sd.V);
                useNet = mf.w > 0.f && sd.frontFacing && wiL.z > 0.f;
            }
            if (__any_sync(0xFFFFFFFFu, useNet)) {
                const int lane = threadIdx.x & 31;
                float x[mlp::kIn];
                mlp::featureRow(wiL.x, wiL.y, wiL.z, wavelength, mf, x);
                uint32_t* row = reinterpret_cast<uint32_t*>(wbuf + lane * mlp::kSWH);
#pragma unroll
                for (int k = 0; k < mlp::kIn; k += 2) row[k / 2] = useNet ? mlp::packBf(x[k], x[k + 1]) : 0u;
                __syncwarp();
                mlp::warpForward32InPlace(wbuf, *reinterpret_cast<const mlp::SmemNet*>(ptSmem));
                if (useNet) mlp::packMixture(reinterpret_cast<const float*>(wbuf) + lane * (mlp::kSWH / 2), mix);
                __syncwarp();
            }
        }
        if (hit) {
            const f3 wi = -dir;
            f3 wo = mk3(0.f, 0.f, 0.f);
            float spdf = 0.f, sweight = 0.f, warp = 1.f;
            uint32_t slobe = 0;
            if (!shouldEnd) {
                const DevMaterial* __restrict__ m = P.mats + mid;
                const uint32_t type = __ldg(&m->type);
                // primary sample of the direction: from the proposal (probability c) or uniform
                f2 uw = kNoWarp;
                float mpss = 1.f;
                bool inside = true;
                if (LEARNED && useNet) {
                    const float cl = P.propProb;
                    if (sg.next1D() < cl) {
                        const float u0 = sg.next1D(), u1 = sg.next1D(), u2 = sg.next1D();
                        mlp::sampleMixturePacked(mix, u0, u1, u2, uw.x, uw.y);
                        inside = uw.x >= 0.f && uw.x < 1.f && uw.y >= 0.f && uw.y < 1.f;
                    } else {
                        uw.x = sg.next1D();
                        uw.y = sg.next1D();
                    }
                    mpss = inside ? cl * mlp::mixtureDensityPacked(mix, uw.x, uw.y) + (1.f - cl) : 0.f;
                    if (!inside) uw = f2{.5f, .5f};   // finite sampler arithmetic; a non-delta result is dropped below
                }
                bool ok = ptSample(m, type, sd, sg, wavelength, wo, spdf, sweight, slobe, kLobeAll, mk3(0.f, 0.f, 0.f), uw);
                if (LEARNED && useNet && ok && (slobe & kLobeDelta) == 0) {
                    ok = inside && mpss > 0.f;
                    warp = mpss;
                }
                shouldEnd = !ok || spdf == 0.f;
                const float nc = pdf * spdf * thp * rcpThp;
                shouldEnd = shouldEnd || nc < 1e-6f;
            }
            const uint32_t extra = useNet ? kFlagLearned : 0u;
            const bool isDelta = (slobe & kLobeDelta) != 0;
            const bool isDisp = (slobe & (kLobeDispDeltaR | kLobeDispDeltaT)) != 0;
            const bool isRefl = (slobe & kLobeReflection) != 0;
            const bool isMS = (isRefl && (props.x & plt::kPropMwReflective)) || (!isRefl && (props.x & plt::kPropMwTransmissive));
            if (shouldEnd) {
                flags |= kFlagTerminated;
                append(h.prim, h.b1, h.b2, wi, 0u, extra);
            } else {
                weight *= sweight;
                thp *= rcpThp;
                pdf *= spdf;
                wps *= warp;
                if (isDisp) flags |= kFlagDispersive;
                append(h.prim, h.b1, h.b2, wi, slobe, extra);
                ++len;
                lndp = !isDelta ? spdf : lndp;
                const uint32_t msc = isMS ? (flags >> 16) + 1u : 0u;
                flags = (flags & 0xFFFFu) | (msc << 16);
                flags = isDelta ? (flags | kFlagLastDelta) : (flags & ~kFlagLastDelta);
                if (!isDelta) flags &= ~kFlagOnlyDelta;
                org = sd.newRayOrigin(isRefl);
                dir = wo;
                live = len < P.maxBounces + 1;
            }
        }
        if (act) {
            P.sg[pid] = sg.s0; P.sg[n + pid] = sg.s1; P.sg[2 * n + pid] = sg.s2; P.sg[3 * n + pid] = sg.s3;
            stPlane3(P.org, pid, n, org);
            stPlane3(P.dir, pid, n, dir);
            P.weight[pid] = weight;
            P.pdf[pid] = pdf;
            P.thp[pid] = thp;
            P.lndp[pid] = lndp;
            P.pflags[pid] = flags;
            P.plen[pid] = len;
            if constexpr (LEARNED) P.wpss[pid] = wps;
        }
        const uint32_t qpos = warpAggregatedAdd(P.qcount + it + 1, live);
        if (live) qout[qpos] = pid;
    }
    if (overflow) atomicOr(P.status, plt::kStatusStackOverflow);
    unsigned long long r = recorded;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xFFFFFFFFu, r, o);
    if ((threadIdx.x & 31u) == 0 && r) atomicAdd(P.stats, r);
    addTraversalBytes(P, nv, tt);
}

// The analytic tracer's segment kernel: trace, Russian roulette and the sample in one pass per
// lane (no warp-uniform phase for the network), which keeps its register allocation lean.
__global__ void __launch_bounds__(128, PLT_BOUNCE_MIN_BLOCKS) ptBounceAnalyticKernel(const PtParams P, uint32_t it) {
    const uint32_t n = P.npix;
    const uint32_t count = it == 0 ? P.nWave : *((volatile uint32_t*)(P.qcount + it));
    const uint32_t* qin = (it & 1u) ? P.queue0 : P.queue1;
    uint32_t* qout = (it & 1u) ? P.queue1 : P.queue0;
    const float4* nodes = reinterpret_cast<const float4*>(P.nodes);
    uint32_t nv = 0, tt = 0, overflow = 0, recorded = 0;
    const Ctx c{P.profiles, P.nProfiles, P.flags};
    // warps take 32 consecutive positions of the shading order at a time (the queue order when the
    // segment is not sorted)
    uint32_t* next = P.segOrder ? P.segSort + it * plt::kSegSortWords + 2 * plt::kSegKeys : nullptr;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t rr = 0;; ++rr) {
        uint32_t c0 = 0;
        if (next) {
            if (lane == 0) c0 = atomicAdd(next, 32u);
            c0 = __shfl_sync(0xFFFFFFFFu, c0, 0);
        } else {
            c0 = rr * stride + blockIdx.x * blockDim.x + (threadIdx.x & ~31u);
        }
        if (c0 >= count) break;
        const uint32_t pos = c0 + lane;
        const uint32_t slot = next && pos < count ? P.segOrder[pos] : pos;
        bool live = false;
        uint32_t pid = 0;
        if (pos < count) {
            pid = (uint32_t)pltIdx(P.status, it == 0 ? slot : qin[pltIdx(P.status, slot, n, kSiteQueue)], n, kSitePath);
            SampleGen sg;
            sg.s0 = P.sg[pid]; sg.s1 = P.sg[n + pid]; sg.s2 = P.sg[2 * n + pid]; sg.s3 = P.sg[3 * n + pid];
            sg.tiny = (P.opt & plt::kPtTinySg) != 0;
            f3 org = ldPlane3(P.org, pid, n), dir = ldPlane3(P.dir, pid, n);
            float weight = P.weight[pid], pdf = P.pdf[pid], thp = P.thp[pid], lndp = P.lndp[pid];
            uint32_t flags = P.pflags[pid], len = P.plen[pid];
            const float wavelength = P.wl[pid];
            auto append = [&](uint32_t prim, float b1, float b2, f3 wi, uint32_t lobe) {
                len = (uint32_t)pltIdx(P.status, len, (size_t)P.maxBounces + 1, kSiteBounce);
                const size_t o = (size_t)len * n + pid;
                P.bFlags[o] = flags;
                P.bPrim[o] = prim;
                P.bBary[(size_t)len * 2 * n + pid] = b1;
                P.bBary[(size_t)len * 2 * n + n + pid] = b2;
                const f2 e = ndirToOctEqualArea(wi);
                P.bEw[(size_t)len * 2 * n + pid] = e.x;
                P.bEw[(size_t)len * 2 * n + n + pid] = e.y;
                P.bLobe[o] = lobe;
                P.bLndp[o] = lndp;
                P.bContrib[o] = 1.f / (pdf * thp);
                ++recorded;
            };
            for (int guard = 0; guard < 64; ++guard) {
                const TraceResult h = guard == 0 && P.segPrim
                                          ? segmentHit(P, slot)
                                          : traverse<false>(nodes, P.tris, org.x, org.y, org.z, dir.x, dir.y, dir.z, 0.f, kFltMax, nv, tt,
                                                            overflow, __ldg(&P.scenes[sceneOf(P, P.pidBase + pid)].root));
                const f3 wi = -dir;
                if (h.prim == kNoHit) {
                    flags |= kFlagMiss;
                    append(kNoHit, 0.f, 0.f, wi, 0u);
                    break;
                }
                const VData v = vertexData(P, h.prim, h.b1, h.b2);
                const uint32_t mid = (uint32_t)pltIdx(P.status, __ldg(P.triMat + h.prim), P.nMats, kSiteMaterial);
                const uint2 props = __ldg(P.matProps + mid);
                const SD sd = prepareSD(v, props.x, wi);
                if ((props.x & plt::kPropAlphaZero) && (P.opt & plt::kPtAlphaMask)) {   // alpha mask: continue the same ray
                    org = sd.newRayOrigin(false);
                    continue;
                }
                // Russian roulette RR(1 - weight, 2, u) (pltpt.slangh:170-176); pow of a negative
                // base is NaN as in the shader
                float rcpThp = 1.f;
                if (P.opt & plt::kPtDoRR) {
                    const float rrVal = 1.f - weight;
                    const float p = rrVal < 0.f ? __int_as_float(0x7fffffff) : rrVal * rrVal;
                    const float u = sg.next1D();
                    rcpThp = u < p ? 0.f : 1.f - p;
                }
                bool shouldEnd = len == P.maxBounces || (rcpThp == 0.f && len > 0);
                f3 wo = mk3(0.f, 0.f, 0.f);
                float spdf = 0.f, sweight = 0.f;
                uint32_t slobe = 0;
                if (!shouldEnd) {
                    const DevMaterial* __restrict__ m = P.mats + mid;
                    const bool ok = ptSample(m, __ldg(&m->type), sd, sg, wavelength, wo, spdf, sweight, slobe);
                    shouldEnd = !ok || spdf == 0.f;
                    const float nc = pdf * spdf * thp * rcpThp;
                    shouldEnd = shouldEnd || nc < 1e-6f;
                }
                const bool isDelta = (slobe & kLobeDelta) != 0;
                const bool isDisp = (slobe & (kLobeDispDeltaR | kLobeDispDeltaT)) != 0;
                const bool isRefl = (slobe & kLobeReflection) != 0;
                const bool isMS = (isRefl && (props.x & plt::kPropMwReflective)) || (!isRefl && (props.x & plt::kPropMwTransmissive));
                if (shouldEnd) {
                    flags |= kFlagTerminated;
                    append(h.prim, h.b1, h.b2, wi, 0u);
                    break;
                }
                weight *= sweight;
                thp *= rcpThp;
                pdf *= spdf;
                if (isDisp) flags |= kFlagDispersive;
                append(h.prim, h.b1, h.b2, wi, slobe);
                ++len;
                lndp = !isDelta ? spdf : lndp;
                const uint32_t msc = isMS ? (flags >> 16) + 1u : 0u;
                flags = (flags & 0xFFFFu) | (msc << 16);
                flags = isDelta ? (flags | kFlagLastDelta) : (flags & ~kFlagLastDelta);
                if (!isDelta) flags &= ~kFlagOnlyDelta;
                org = sd.newRayOrigin(isRefl);
                dir = wo;
                live = len < P.maxBounces + 1;
                break;
            }
            if (!live && (flags & (kFlagMiss | kFlagTerminated)) == 0) {
                // 64 alpha-masked hits in a row: end the path with an empty terminal record
                flags |= kFlagTerminated;
                append(kNoHit, 0.f, 0.f, -dir, 0u);
            }
            P.sg[pid] = sg.s0; P.sg[n + pid] = sg.s1; P.sg[2 * n + pid] = sg.s2; P.sg[3 * n + pid] = sg.s3;
            stPlane3(P.org, pid, n, org);
            stPlane3(P.dir, pid, n, dir);
            P.weight[pid] = weight;
            P.pdf[pid] = pdf;
            P.thp[pid] = thp;
            P.lndp[pid] = lndp;
            P.pflags[pid] = flags;
            P.plen[pid] = len;
        }
        const uint32_t qpos = warpAggregatedAdd(P.qcount + it + 1, live);
        if (live) qout[qpos] = pid;
    }
    if (overflow) atomicOr(P.status, plt::kStatusStackOverflow);
    unsigned long long r = recorded;
    for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xFFFFFFFFu, r, o);
    if ((threadIdx.x & 31u) == 0 && r) atomicAdd(P.stats, r);
    addTraversalBytes(P, nv, tt);
}

#endif  // PLT_PT_SAMPLE_PASS

// ---- manifold NEE (Manifolds.slangh, DifferentialShadingGeometry.slang) ---------------------
struct F3pdv { f3 v, ddu, ddv; };
struct F3kpdv { f3 v, ddu, ddv, ddl; };
struct DSG {
    F3pdv p, n, s, t;
    PLT_DI f3 fromLocal(f3 v) const { return s.v * v.x + t.v * v.y + n.v * v.z; }
    PLT_DI F3pdv pdw(f3 dst) const {
        F3pdv w;
        w.v = dst - p.v;
        const float ilo = 1.f / sqrtf(dot(w.v, w.v));
        w.v = w.v * ilo;
        w.ddu = (p.ddu - w.v * dot(w.v, p.ddu)) * -ilo;
        w.ddv = (p.ddv - w.v * dot(w.v, p.ddv)) * -ilo;
        return w;
    }
};
PLT_DI f3 zero3() { return mk3(0.f, 0.f, 0.f); }
// differentialShadingGeometry, DifferentialShadingGeometry.slang:94-178 (untextured meshes: the
// (1,0), (0,1) triangle parameterisation, so dp/du = p1 - p0 and dp/dv = p2 - p0)
PLT_NI DSG differentialShadingGeometry(const PtParams& P, uint32_t prim, float b1, float b2) {
    const float w0 = 1.f - b1 - b2;
    const uint32_t i0 = __ldg(P.idx + 3 * prim), i1 = __ldg(P.idx + 3 * prim + 1), i2 = __ldg(P.idx + 3 * prim + 2);
    const f3 p0 = ld3s(P.pos, i0), p1 = ld3s(P.pos, i1), p2 = ld3s(P.pos, i2);
    const f3 n0 = ld3s(P.nrm, i0), n1 = ld3s(P.nrm, i1), n2 = ld3s(P.nrm, i2);
    DSG g;
    g.p.v = p0 * w0 + p1 * b1 + p2 * b2;
    g.n.v = n0 * w0 + n1 * b1 + n2 * b2;
    const float il = 1.0f / sqrtf(dot(g.n.v, g.n.v));
    g.n.v = g.n.v * il;
    g.n.ddu = (n1 - n0) * il;
    g.n.ddv = (n2 - n0) * il;
    g.n.ddu = g.n.ddu - g.n.v * dot(g.n.v, g.n.ddu);
    g.n.ddv = g.n.ddv - g.n.v * dot(g.n.v, g.n.ddv);
    g.p.ddu = p1 - p0;
    g.p.ddv = p2 - p0;
    g.s.v = g.p.ddu - g.n.v * dot(g.n.v, g.p.ddu);
    float ils = 1.0f / sqrtf(dot(g.s.v, g.s.v));
    g.s.v = g.s.v * ils;
    if (g.p.ddu.x == 0.f && g.p.ddu.y == 0.f && g.p.ddu.z == 0.f) {
        g.s.v = perp_stark(g.n.v);
        ils = 1.0f;
    }
    g.t.v = cross(g.n.v, g.s.v);
    g.s.ddu = ((-g.n.ddu) * dot(g.n.v, g.p.ddu) - g.n.v * dot(g.n.ddu, g.p.ddu)) * ils;
    g.s.ddv = ((-g.n.ddv) * dot(g.n.v, g.p.ddu) - g.n.v * dot(g.n.ddv, g.p.ddu)) * ils;
    g.s.ddu = g.s.ddu - g.s.v * dot(g.s.ddu, g.s.v);
    g.s.ddv = g.s.ddv - g.s.v * dot(g.s.ddv, g.s.v);
    g.t.ddu = cross(g.n.ddu, g.s.v) + cross(g.n.v, g.s.ddu);
    g.t.ddv = cross(g.n.ddv, g.s.v) + cross(g.n.v, g.s.ddv);
    return g;
}
// reflectDerivatives / refractDerivatives, DifferentialShadingGeometry.slang:180-222
PLT_DI F3kpdv reflectDerivatives(const F3pdv& wi, const F3pdv& n) {
    const float wn = dot(wi.v, n.v);
    const float dwdun = dot(wi.ddu, n.v), dwdvn = dot(wi.ddv, n.v);
    const float dnduw = dot(n.ddu, wi.v), dndvw = dot(n.ddv, wi.v);
    F3kpdv r;
    r.v = n.v * (2.f * wn) - wi.v;
    r.ddu = (n.v * (dwdun + dnduw) + n.ddu * wn) * 2.f - wi.ddu;
    r.ddv = (n.v * (dwdvn + dndvw) + n.ddv * wn) * 2.f - wi.ddv;
    r.ddl = zero3();
    return r;
}
PLT_DI F3kpdv refractDerivatives(const F3pdv& wi, F3pdv n, float eta) {
    const float wn = dot(wi.v, n.v);
    eta = wn < 0.f ? eta : 1.f / eta;
    if (wn < 0.f) { n.v = -n.v; n.ddu = -n.ddu; n.ddv = -n.ddv; }
    const float eta2 = eta * eta;
    const float dwdun = dot(wi.ddu, n.v), dwdvn = dot(wi.ddv, n.v);
    const float dnduw = dot(n.ddu, wi.v), dndvw = dot(n.ddv, wi.v);
    const float root = sqrtf(fmaxf(0.f, 1.f - eta2 * (1.0f - wn * wn)));
    F3kpdv r;
    if (root == 0.f) { r.v = r.ddu = r.ddv = r.ddl = zero3(); return r; }
    const float a = eta - eta2 * wn / root;
    r.v = (wi.v - n.v * wn) * -eta - n.v * root;
    r.ddu = n.v * (a * (dnduw + dwdun)) + n.ddu * (eta * wn - root) - wi.ddu * eta;
    r.ddv = n.v * (a * (dndvw + dwdvn)) + n.ddv * (eta * wn - root) - wi.ddv * eta;
    r.ddl = zero3();
    return r;
}
// DiffractionGrating.partialDerivatives, DiffractionGrating.slang:188-265
PLT_NI F3kpdv gratingDerivatives(const DSG& g, const F3pdv& wi, float gx, float gy, float ipx, float ipy, int lx, int ly, float wavelength) {
    F3kpdv ret;
    ret.v = ret.ddu = ret.ddv = ret.ddl = zero3();
    const F3pdv& n = g.n;
    const f3 Xv = g.fromLocal(mk3(gx, gy, 0.f));
    const f3 Xdu = g.s.ddu * gx + g.t.ddu * gy, Xdv = g.s.ddv * gx + g.t.ddv * gy;
    const float lambda = 1e-3f * wavelength;
    const float lpx = (float)lx * ipx, lpy = (float)ly * ipy;
    const f3 Y = cross(n.v, Xv);
    const float x = dot(wi.v, Xv), y = dot(wi.v, Y), z = dot(wi.v, n.v);
    const float px = sqrtf(x * x + z * z), py = sqrtf(y * y + z * z);
    const float iqx = px > kFltEps ? 1.f / px : 0.f, iqy = py > kFltEps ? 1.f / py : 0.f;
    const float a = lambda * lpx - x * iqx, b = lambda * lpy - y * iqy;
    const float oneMinusA2 = fmaxf(0.f, 1 - a * a);
    const float m = -oneMinusA2 / ((a * b) * (a * b) - 1);
    const float q = 1 - b * b * m;
    if (a > 1.f || a < -1.f || b > 1.f || b < -1.f || q < 0.f || !(m >= 0.f)) return ret;
    const float sqrtOneM = sqrtf(q), sqrtM = sqrtf(m);
    const float c = .5f / (sqrtOneM * sqrtf(oneMinusA2));
    const float dxdu = dot(wi.v, Xdu) + dot(wi.ddu, Xv), dxdv = dot(wi.v, Xdv) + dot(wi.ddv, Xv);
    const float dzdu = dot(wi.v, n.ddu) + dot(wi.ddu, n.v), dzdv = dot(wi.v, n.ddv) + dot(wi.ddv, n.v);
    const float iqx3 = iqx * iqx * iqx, iqy3 = iqy * iqy * iqy;
    const float dadu = z * (x * dzdu - z * dxdu) * iqx3, dbdu = z * (y * dzdu - z * dxdu) * iqy3;
    const float dadv = z * (x * dzdv - z * dxdv) * iqx3, dbdv = z * (y * dzdv - z * dxdv) * iqy3;
    const float den = ((a * b) * (a * b) - 1) * ((a * b) * (a * b) - 1);
    const float dmdu = 2 * a * (a * b * oneMinusA2 * dbdu - dadu * (1 - b * b)) / den;
    const float dmdv = 2 * a * (a * b * oneMinusA2 * dbdv - dadv * (1 - b * b)) / den;
    const float dmdl = 2 * a * (a * b * oneMinusA2 * lpy - lpx * (1 - b * b)) / den;
    ret.v = Xv * (a * sqrtOneM) + Y * (b * sqrtM) + n.v * sqrtf(fmaxf(0.f, 1 - a * a * q - b * b * m));
    auto d = [&](float da, float db, float dm) {
        return Xv * ((q * da - a * b * (b * dm / 2.f + m * db)) / sqrtOneM) + Y * ((b * dm / 2.f + m * db) / sqrtM) +
               n.v * ((-2 * a * da * q - b * (b * dm + 2.f * m * db) + a * a * b * (b * dm + 2.f * m * db)) * c);
    };
    ret.ddu = d(dadu, dbdu, dmdu);
    ret.ddv = d(dadv, dbdv, dmdv);
    ret.ddl = d(lpx, lpy, dmdl);
    return ret;
}
// IMaterialInstance.partialDerivatives of the PLT*BSDF.slang wrappers (world space)
PLT_DI F3kpdv ptPartialDerivatives(const DevMaterial* __restrict__ m, uint32_t type, const F3pdv& wi, const DSG& g, uint32_t lobe,
                                   float wavelength) {
    switch (type) {
    case kMatDielectric:
        if (lobe & kLobeTransmission) return refractDerivatives(wi, g.n, dielIor(m->p, kOfWl(wavelength)));
        return reflectDerivatives(wi, g.n);
    case kMatThin:
        if (lobe & kLobeTransmission) {
            F3kpdv r;
            r.v = -wi.v; r.ddu = -wi.ddu; r.ddv = -wi.ddv; r.ddl = zero3();
            return r;
        }
        return reflectDerivatives(wi, g.n);
    case kMatGratedConductor:
    case kMatGratedOpaque: {
        int lx, ly;
        decodeGratingLobe(lobe, lx, ly);
        if (lx == 0 && ly == 0) return reflectDerivatives(wi, g.n);
        return gratingDerivatives(g, wi, __ldg(m->p + PD_GX), __ldg(m->p + PD_GY), __ldg(m->p + PD_IPX), __ldg(m->p + PD_IPY), lx, ly,
                                  wavelength);
    }
    case kMatDiffuse: {
        F3kpdv r;
        r.v = r.ddu = r.ddv = r.ddl = zero3();
        return r;
    }
    default: return reflectDerivatives(wi, g.n);
    }
}
// manifoldOneStep with sphcoords and their derivatives, Manifolds.slangh:283-347
PLT_DI void sphcoords(f3 w, float& theta, float& phi) {
    theta = acosf(fminf(fmaxf(w.z, -1.f), 1.f));
    phi = atan2f(w.y, w.x);
    phi += phi < 0.f ? k2Pi : 0.f;
}
PLT_DI bool manifoldOneStep(const F3pdv& w, const F3kpdv& ws, const F3pdv& p, float& lenC, f3& stepDir) {
    float t0, p0, t1, p1;
    sphcoords(w.v, t0, p0);
    sphcoords(ws.v, t1, p1);
    const float dt = t0 - t1;
    float dp = p0 - p1;
    dp = fabsf(dp) > kPi ? dp - signf(dp) * k2Pi : dp;
    lenC = sqrtf(dt * dt + dp * dp);
    const float aO = -1.f / sqrtf(fmaxf(0.f, 1.f - w.v.z * w.v.z)), iO = 1.f / (w.v.x * w.v.x + w.v.y * w.v.y);
    const float aI = -1.f / sqrtf(fmaxf(0.f, 1.f - ws.v.z * ws.v.z)), iI = 1.f / (ws.v.x * ws.v.x + ws.v.y * ws.v.y);
    const float A = aO * w.ddu.z - aI * ws.ddu.z;
    const float B = aO * w.ddv.z - aI * ws.ddv.z;
    const float C = iO * (w.v.x * w.ddu.y - w.v.y * w.ddu.x) - iI * (ws.v.x * ws.ddu.y - ws.v.y * ws.ddu.x);
    const float D = iO * (w.v.x * w.ddv.y - w.v.y * w.ddv.x) - iI * (ws.v.x * ws.ddv.y - ws.v.y * ws.ddv.x);
    const float det = A * D - B * C;
    if (fabsf(det) < 4e-6f) return false;      // tryInvert, MathHelpers.slang:484-498
    const float id = 1.0f / det;
    const float dx = (D * id) * dt + (-B * id) * dp, dy = (-C * id) * dt + (A * id) * dp;
    stepDir = p.ddu * dx + p.ddv * dy;
    return true;
}

constexpr int kMaxMsOccluders = 4;
struct MSHit {
    uint32_t prim, lobe;
    float b1, b2;
    f3 posW;
};
struct MSData {
    MSHit hits[kMaxMsOccluders];
    f3 woLastHitToLight;
    int hitCount;
    uint32_t iterations;
    float wavelength, pdf;
    bool dispersive;
};
struct TraceCounters {
    uint32_t nv, tt, overflow, shadowRays;
};
// closest-hit shadow ray (ShadowRays.slangh:96-135): a hit needs dist > 0
PLT_DI bool shadowRayClosest(const PtParams& P, int32_t root, f3 o, f3 d, float tmin, float tmax, TraceResult& h, TraceCounters& tc) {
    ++tc.shadowRays;
    h = traverse<false>(reinterpret_cast<const float4*>(P.nodes), P.tris, o.x, o.y, o.z, d.x, d.y, d.z, tmin, tmax, tc.nv, tc.tt, tc.overflow,
                        root);
    return h.prim != kNoHit && h.t > 0.f;
}
// manifoldSampleVertex, Manifolds.slangh:84-108
PLT_DI bool manifoldSampleVertex(const PtParams& P, uint32_t prim, float b1, float b2, const SD& sd, uint32_t mid, f3 lightDir,
                                 SampleGen& sg, MSData& d) {
    const DevMaterial* __restrict__ m = P.mats + mid;
    f3 wo;
    float pdf = 0.f, weight = 0.f;
    uint32_t lobe = 0;
    if (!ptSample(m, __ldg(&m->type), sd, sg, d.wavelength, wo, pdf, weight, lobe, kLobeDelta, lightDir)) return false;
    d.pdf *= pdf;
    MSHit& h = d.hits[d.hitCount];
    h.prim = prim;
    h.b1 = b1;
    h.b2 = b2;
    h.posW = sd.posW;
    h.lobe = lobe;
    d.dispersive = d.dispersive || (lobe & (kLobeDispDeltaR | kLobeDispDeltaT)) != 0;
    ++d.hitCount;
    return true;
}
// traceMNEEOccluders, Manifolds.slangh:110-160: the closest-hit shadow ray towards the light and a
// hinted delta sample at every occluder (the only random draws of a manifold sample).  Returns
// kMsFail (no contribution), kMsVisible (no occluder: the light is visible) or kMsWalk (occluders
// recorded in d; manifoldWalk completes the sample).
constexpr int kMsFail = 0, kMsVisible = 1, kMsWalk = 2;
PLT_NI int manifoldOccluders(const PtParams& P, int32_t root, f3 rayO, f3 rayD, float tmax, int maxMS, SampleGen& sg, MSData& d,
                             TraceCounters& tc) {
    const int maxOcc = (int)min(P.mneeMaxOccluders, (uint32_t)kMaxMsOccluders);
    const f3 wi = -rayD;
    for (int guard = 0; guard <= kMaxMsOccluders; ++guard) {
        TraceResult h;
        if (!shadowRayClosest(P, root, rayO, rayD, 0.f, tmax, h, tc)) break;
        if (d.hitCount >= maxOcc || d.hitCount >= maxMS) return kMsFail;
        VData v = vertexData(P, h.prim, h.b1, h.b2);
        v.posW = rayO + rayD * h.t;
        const uint32_t mid = __ldg(P.triMat + h.prim);
        const uint2 props = __ldg(P.matProps + mid);
        const SD sd = prepareSD(v, props.x, wi);
        if (!(props.x & plt::kPropMwTransmissive)) return kMsFail;
        if (!manifoldSampleVertex(P, h.prim, h.b1, h.b2, sd, mid, -wi, sg, d) || (d.hits[d.hitCount - 1].lobe & kLobeTransmission) == 0)
            return kMsFail;
        rayO = newRayOriginToward(sd, rayD);
        tmax -= h.t;
    }
    return d.hitCount == 0 ? kMsVisible : kMsWalk;
}
// manifoldNEESample's walk, Manifolds.slangh:162-281: Newton steps on the spherical-angle
// constraint of every occluder with re-projection onto the same geometry instance, then the
// visibility of the light from the last vertex.  Deterministic (no random draws).
PLT_NI bool manifoldWalk(const PtParams& P, int32_t root, f3 origin, f3 lightPos, f3 lightDir, bool distant, MSData& d,
                         TraceCounters& tc) {
    float beta[kMaxMsOccluders];
#pragma unroll
    for (int i = 0; i < kMaxMsOccluders; ++i) beta[i] = 1.f;
    bool success = false;
    while (!success) {
        success = true;
        for (int idx = 0; idx < d.hitCount; ++idx) {
            MSHit& h = d.hits[idx];
            const uint32_t mid = __ldg(P.triMat + h.prim);
            const DSG g = differentialShadingGeometry(P, h.prim, h.b1, h.b2);
            const f3 p0 = idx == 0 ? origin : d.hits[idx - 1].posW;
            const F3pdv pdv0 = g.pdw(p0);
            const f3 p2 = idx + 1 == d.hitCount ? lightPos : d.hits[idx + 1].posW;
            // a distant light fixes the direction towards it at every vertex of the chain
            // (Manifolds.slangh:199-202)
            F3pdv pdv2;
            if (distant) {
                pdv2.v = lightDir;
                pdv2.ddu = mk3(0.f, 0.f, 0.f);
                pdv2.ddv = mk3(0.f, 0.f, 0.f);
            } else {
                pdv2 = g.pdw(p2);
            }
            const bool woIsIn = dot(pdv2.v, g.n.v) < 0.f;
            const F3pdv wiP = woIsIn ? pdv0 : pdv2;
            const F3pdv woP = woIsIn ? pdv2 : pdv0;
            const DevMaterial* __restrict__ m = P.mats + mid;
            const F3kpdv wos = ptPartialDerivatives(m, __ldg(&m->type), wiP, g, h.lobe, d.wavelength);
            if (wos.v.x == 0.f && wos.v.y == 0.f && wos.v.z == 0.f) return false;
            float lenC;
            f3 stepDir;
            if (!manifoldOneStep(woP, wos, g.p, lenC, stepDir)) return false;
            if (lenC < P.mneeThreshold) continue;
            success = false;
            for (;;) {
                if (++d.iterations > P.mneeMaxIterations) return false;
                const f3 proposal = h.posW - stepDir * beta[idx];
                f3 dirTo = proposal - p0;
                const float dist = sqrtf(dot(dirTo, dirTo));
                dirTo = dirTo / dist;
                TraceResult hp;
                const bool hit = shadowRayClosest(P, root, p0, dirTo, fmaxf(1e-4f, .99f * dist), 1.01f * dist, hp, tc);
                if (!hit || __ldg(P.triInst + h.prim) != __ldg(P.triInst + hp.prim)) {
                    beta[idx] /= 4.f;
                    continue;
                }
                h.prim = hp.prim;
                h.b1 = hp.b1;
                h.b2 = hp.b2;
                h.posW = p0 + dirTo * hp.t;
                beta[idx] = fminf(1.0f, 2.f * beta[idx]);
                break;
            }
        }
    }
    const f3 pl = d.hits[d.hitCount - 1].posW;
    f3 dir;
    float dist;
    if (!distant) {
        dir = lightPos - pl;
        dist = sqrtf(dot(dir, dir));
        dir = dir / dist;
    } else {
        dir = lightDir;
        dist = kFltMax;
    }
    ++tc.shadowRays;
    const TraceResult vis = traverse<true>(reinterpret_cast<const float4*>(P.nodes), P.tris, pl.x, pl.y, pl.z, dir.x, dir.y, dir.z, 1e-4f,
                                           dist, tc.nv, tc.tt, tc.overflow, root);
    d.woLastHitToLight = dir;
    return vis.prim == kNoHit;
}

// ---- solve pass -----------------------------------------------------------------------------
// A deferred manifold walk: everything the walk and the rest of its NEE sample need (the light
// sample, the occluder search's result, the replay's origin).  The solve kernel records one per
// NEE sample that found occluders; ptMneeKernel finishes them as a dense wavefront.
template <int H> struct MneeTask {
    MSData ms;
    f3 tposW, ldir, msOrigin;
    float ldist, tpdf;
    float srcSize;                // the sourced beam's area (area lights) or solid angle (distant lights)
    float Le[H], swl[H];
    uint32_t pid, p, curMS;
};

template <int H> struct Bnc {
    uint32_t prim, lobe, flags;
    float b1, b2, contrib, lndp;
    f3 wi;
};
template <int H> PLT_DI Bnc<H> readBounce(const PtParams& P, uint32_t pid, int p) {
    const uint32_t n = P.npix;
    pid = (uint32_t)pltIdx(P.status, pid, n, kSitePath);
    p = (int)pltIdx(P.status, (size_t)p, (size_t)P.maxBounces + 1, kSiteBounce);
    const size_t o = (size_t)p * n + pid;
    Bnc<H> b;
    b.prim = P.bPrim[o];
    b.lobe = P.bLobe[o];
    b.flags = P.bFlags[o];
    b.b1 = P.bBary[(size_t)p * 2 * n + pid];
    b.b2 = P.bBary[(size_t)p * 2 * n + n + pid];
    b.contrib = P.bContrib[o];
    b.lndp = P.bLndp[o];
    b.wi = octToNdirEqualArea(f2{P.bEw[(size_t)p * 2 * n + pid], P.bEw[(size_t)p * 2 * n + n + pid]});
    return b;
}

// ---- debug views (pltpt_debug.slangh, DebugViewType.slangh) ------------------------------------
#define PLT_COLOUR_MAP_STORAGE static __constant__ const
#include "plt_colour_maps.h"

// A path's debug colour: the sum of the values written by the selected view, and their count.
struct DebugAcc {
    float r, g, b, n;
};
// writeDebugOutput: added when the view is the selected one and the value is finite
PLT_DI void dbgWrite(DebugAcc* d, uint32_t selected, uint32_t view, f3 v) {
    if (d && selected == view && isfinite(v.x) && isfinite(v.y) && isfinite(v.z)) {
        d->r += v.x;
        d->g += v.y;
        d->b += v.z;
        d->n += 1.f;
    }
}
// ccMagma / ccInferno (RenderPasses/PLTPT/ColourCoding.slang): lerp between the bins around
// val * 256, both clamped to [0, 255] (a non-finite val gives a non-finite colour, never written)
PLT_DI f3 colourCode(const float (*t)[3], float val) {
    val *= 256.f;
    if (!isfinite(val)) return mk3(val - val, 0.f, 0.f);
    const int l = (int)fminf(fmaxf(val, 0.f), 255.f), h = (int)fminf(fmaxf(val + 1.f, 0.f), 255.f);
    const float fr = val - floorf(val);
    const f3 a = mk3(t[l][0], t[l][1], t[l][2]), b = mk3(t[h][0], t[h][1], t[h][2]);
    return a + (b - a) * fr;
}
// PLTBeam.coherenceArea(k) = pi sqrt(1 / det(invTheta(k))) and coherenceAnisotropy(k) =
// 1 - S00 / S11 of svd_symmetric(invTheta(k)) (PLT.slang:57-64,186-197; MathHelpers.slang:583-605)
template <int H> PLT_DI void coherenceDebug(const DBeam<H>& b, float k, float& area, float& aniso) {
    const float rmm = b.r_m * 1e+3f;
    const float s = (k / k2Pi / rmm) * (k / k2Pi / rmm);
    const float a = s * b.D0, c = s * b.D1, d = s * b.D2;
    area = kPi * sqrtf(1.f / (a * d - c * c));
    const float a2 = a * a, b2 = c * c, c2 = c * c, d2 = d * d;
    const float y = 2.f * a * c + 2.f * c * d, x = a2 + b2 - c2 - d2;
    const float s1 = a2 + b2 + c2 + d2, s2 = sqrtf(x * x + y * y);
    aniso = 1.f - sqrtf((s1 + s2) / 2.f) / sqrtf((s1 - s2) / 2.f);
}

// One vertex of a forward replay: the beam propagated to the vertex (at msPos for a manifold
// vertex) and replaced by the BSDF's response towards qwo, with the lambda pdfs of spectral MIS
// (the body of forwardUnwind / manifoldForwardUnwind, pltpt_solve.rt.slang:48-93).
template <int H>
PLT_DI void replayVertex(const PtParams& P, uint32_t qprim, float qb1, float qb2, f3 qwo, uint32_t qlobe, bool msVertex, f3 msPos,
                         PBeam<H>& pb, const Ctx& c, bool hwssMis, uint32_t& evals) {
    VData qv = vertexData(P, qprim, qb1, qb2);
    if (msVertex) qv.posW = msPos;
    const uint32_t qmid = __ldg(P.triMat + qprim);
    const SD qsd = prepareSD(qv, __ldg(P.matProps + qmid).x, -pb.b.r);
    propagate(pb, qsd.posW);
    const DevMaterial* __restrict__ qm = P.mats + qmid;
    const uint32_t qtype = __ldg(&qm->type);
    ptEval<H>(qm, qtype, c, qsd, qwo, qlobe, pb.b);
    ++evals;
    if (hwssMis) {
        float lp[H];
        ptLambdaPdf<H>(qm, qtype, qsd, qwo, qlobe, pb.b, lp);
#pragma unroll
        for (int j = 0; j < H; ++j) pb.spdf[j] *= lp[j];
    }
}

template <int H>
PLT_DI void replayFinish(const PtParams& P, const PtScene& S, int p, const Bnc<H>& bounce, PBeam<H>& pb, bool hwssMis, float& Lr, float& Lg,
                         float& Lb, DebugAcc* dbg);

// Forward replay of one beam source of vertex p and its measurement (pltpt_solve.rt.slang:48-147):
// the manifold vertices (last to first, manifoldForwardUnwind :80-93), the current vertex (NEE,
// non-delta lobes), then vertices p-1 .. 0, the camera polariser and spectrumToRgb.  Adds the
// path's contribution to (Lr, Lg, Lb).
template <int H>
PLT_DI void replayMeasure(const PtParams& P, const PtScene& S, uint32_t pid, int p, const Bnc<H>& bounce, PBeam<H>& pb, const MSData& ms,
                          int nMs, f3 msOrigin, bool evalCurrent, const Ctx& c, bool hwssMis, float& Lr, float& Lg, float& Lb,
                          uint32_t& evals, DebugAcc* dbg = nullptr) {
    // forward replay: the manifold vertices (last to first, manifoldForwardUnwind,
    // pltpt_solve.rt.slang:80-93), the current vertex (NEE, non-delta lobes), then p-1 .. 0
    const int total = nMs + (evalCurrent ? 1 : 0) + p;
    for (int k = 0; k < total; ++k) {
        uint32_t qprim, qlobe;
        float qb1, qb2;
        f3 qwo;
        bool msVertex = false;
        f3 msPos;
        if (k < nMs) {
            const int idx = nMs - 1 - k;
            const MSHit& h = ms.hits[idx];
            qprim = h.prim; qlobe = h.lobe; qb1 = h.b1; qb2 = h.b2;
            msPos = h.posW;
            msVertex = true;
            const f3 p2 = idx == 0 ? msOrigin : ms.hits[idx - 1].posW;
            qwo = normalize(p2 - h.posW);
        } else if (evalCurrent && k == nMs) {
            qprim = bounce.prim; qlobe = kLobeNonDelta; qb1 = bounce.b1; qb2 = bounce.b2; qwo = bounce.wi;
        } else {
            const int q = p - 1 - (k - nMs - (evalCurrent ? 1 : 0));
            const Bnc<H> bq = readBounce<H>(P, pid, q);
            qprim = bq.prim; qlobe = bq.lobe; qb1 = bq.b1; qb2 = bq.b2; qwo = bq.wi;
        }
        replayVertex<H>(P, qprim, qb1, qb2, qwo, qlobe, msVertex, msPos, pb, c, hwssMis, evals);
    }
    replayFinish<H>(P, S, p, bounce, pb, hwssMis, Lr, Lg, Lb, dbg);
}

// The measurement that ends a forward replay (pltpt_solve.rt.slang:96-147): the beam propagated to
// the camera, the camera polariser, spectral MIS or the component count, spectrumToRgb; adds the
// contribution to (Lr, Lg, Lb).
template <int H>
PLT_DI void replayFinish(const PtParams& P, const PtScene& S, int p, const Bnc<H>& bounce, PBeam<H>& pb, bool hwssMis, float& Lr, float& Lg,
                         float& Lb, DebugAcc* dbg) {
    // measure (no camera polarizer unless set)
    if (!(P.opt & plt::kPtUseDirect) && p <= 1) return;
    if (dbg) {
        // coherence views, before the propagation to the camera (pltpt_solve.rt.slang:102-106)
        float area, aniso;
        coherenceDebug<H>(pb.b, k2Pi / (1e-3f * pb.b.wl[0]), area, aniso);
        dbgWrite(dbg, P.debugView, PLT_DEBUG_VIEW_COHERENCE_AREA, colourCode(kMagma, sqrtf(area) / 150.f));
        dbgWrite(dbg, P.debugView, PLT_DEBUG_VIEW_COHERENCE_ANISOTROPY, colourCode(kInferno, aniso));
    }
    propagate(pb, camPos(S));
    if (S.cam.polarizer > 0.f) {
        const f3 Wc = rnormalize(mk3(S.cam.w[0], S.cam.w[1], S.cam.w[2]));
        const f3 Uc = rnormalize(mk3(S.cam.u[0], S.cam.u[1], S.cam.u[2]));
        pb.b.rotateFrame(Uc, -Wc);
        const float pi = S.cam.polarizer;
        float sth, cth;
        sincosf(S.cam.polarizer_theta, &sth, &cth);
        const float Pm[4][4] = {{.5f, .5f * cth, .5f * sth, 0.f}, {.5f * cth, .5f * (cth * cth), .5f * (cth * sth), 0.f},
                                {.5f * sth, .5f * (cth * sth), .5f * (sth * sth), 0.f}, {0.f, 0.f, 0.f, 0.f}};
#pragma unroll
        for (int j = 0; j < H; ++j) {
            const float in[4] = {pb.b.L[0][j], pb.b.L[1][j], pb.b.L[2][j], pb.b.L[3][j]};
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                float acc = 0.f;
#pragma unroll
                for (int cc = 0; cc < 4; ++cc) acc += ((1.f - pi) * (r == cc ? 1.f : 0.f) + pi * Pm[r][cc]) * in[cc];
                pb.b.L[r][j] = acc;
            }
        }
    }
    float contrib = bounce.contrib;
    if (hwssMis) {
        float sum = 0.f;
#pragma unroll
        for (int j = 0; j < H; ++j) sum += pb.spdf[j];
        contrib *= sum > kFltEps ? pb.spdf[0] / sum : 0.f;
    } else {
        contrib *= 1.f / float(pb.comps);
    }
    float Li[H];
#pragma unroll
    for (int j = 0; j < H; ++j) Li[j] = pb.b.L[0][j];
    const f3 rgb = spectrumToRgb<H>(Li, pb.b.wl, pb.comps);
    const float r = fmaxf(0.f, rgb.x * contrib), g = fmaxf(0.f, rgb.y * contrib), bb = fmaxf(0.f, rgb.z * contrib);
    if (isfinite(r) && isfinite(g) && isfinite(bb)) { Lr += r; Lg += g; Lb += bb; }
    if (dbg) {
        // markDebug (pltpt_debug.slangh:31-50): NaNs and infinities of the path's sum, path length,
        // spectral samples carried, and the polarisation of the hero wavelength at the sensor
        if (isnan(Lr) || isnan(Lg) || isnan(Lb)) dbgWrite(dbg, P.debugView, PLT_DEBUG_VIEW_NANS, mk3(5.f, 0.f, 3.f));
        if (isinf(Lr) || isinf(Lg) || isinf(Lb)) dbgWrite(dbg, P.debugView, PLT_DEBUG_VIEW_INFS, mk3(2.f, 0.f, 5.f));
        dbgWrite(dbg, P.debugView, PLT_DEBUG_VIEW_PATH_LENGTH, colourCode(kMagma, (float)p / (float)(P.maxBounces - 1)));
        dbgWrite(dbg, P.debugView, PLT_DEBUG_VIEW_HWSS_COMPS, colourCode(kMagma, (float)pb.comps / (float)H));
        const float S0 = pb.b.L[0][0], S1 = pb.b.L[1][0], S2 = pb.b.L[2][0], S3 = pb.b.L[3][0];
        const float cp = sqrtf(S3 * S3) / S0, lp = sqrtf(S1 * S1 + S2 * S2) / S0;
        const float lpd = .5f * atan2f(S2, S1);
        const float cl = cosf(lpd), sl = sinf(lpd);
        dbgWrite(dbg, P.debugView, PLT_DEBUG_VIEW_POLARIZATION, mk3(lp * (cl * cl), cp, lp * (sl * sl)));
    }
}

// replayMeasure called out of line from the solve kernel: with deferred replays it runs only for
// manifold samples walked inline, a full replay queue and debug views, so its code stays out of the
// solve kernel's hot instruction stream.
template <int H>
__device__ __noinline__ void replayInline(const PtParams& P, const PtScene& S, uint32_t pid, int p, const Bnc<H>& bounce, PBeam<H>& pb,
                                          const MSData& ms, int nMs, f3 msOrigin, bool evalCurrent, const Ctx& c, bool hwssMis,
                                          float& Lr, float& Lg, float& Lb, uint32_t& evals, DebugAcc* dbg) {
    replayMeasure<H>(P, S, pid, p, bounce, pb, ms, nMs, msOrigin, evalCurrent, c, hwssMis, Lr, Lg, Lb, evals, dbg);
}

// sampleLight for analytic lights (Rendering/Lights/LightHelpers.slang:71-289): the direction and
// distance to the light, the incident radiance already divided by the pdf (Li, at the sampled
// wavelengths wl) and the solid-angle pdf (0 for point and directional lights).  False when the
// light yields no sample (an area light seen from behind).
template <int H>
PLT_DI bool sampleAnalytic(const PtParams& P, const plt::AnalyticLightDev& L, f3 p, float wavelength, SampleGen& sg, bool importance,
                           f3& dir, float& dist, float* Li, float* wl, float& pdf) {
    const uint32_t type = L.type;
    if (type == PLT_LIGHT_POINT) {
        const f3 toLight = mk3(L.pos[0], L.pos[1], L.pos[2]) - p;
        const float distSqr = fmaxf(dot(toLight, toLight), 1e-9f);
        dist = sqrtf(distSqr);
        dir = toLight / dist;
        const float cosTheta = -dot(dir, mk3(L.dir[0], L.dir[1], L.dir[2]));
        float falloff = 1.f;
        if (cosTheta < L.cosOpeningAngle) {
            falloff = 0.f;
        } else if (L.penumbraAngle > 0.f) {
            const float delta = L.openingAngle - acosf(cosTheta);
            const float t = clampf(delta / L.penumbraAngle, 0.f, 1.f);
            falloff = t * t * (3.f - 2.f * t);
        }
        sampleSpectrum<H>(P, L.spectrumId, wavelength, sg, importance, Li, wl);
#pragma unroll
        for (int j = 0; j < H; ++j) Li[j] *= falloff / distSqr;
        pdf = 0.f;
        return true;
    }
    if (type == PLT_LIGHT_DIRECTIONAL) {
        dist = kFltMax;
        dir = -mk3(L.dir[0], L.dir[1], L.dir[2]);
        sampleSpectrum<H>(P, L.spectrumId, wavelength, sg, importance, Li, wl);
        pdf = 0.f;
        return true;
    }
    const float ux = sg.next1D();
    const float uy = sg.next1D();
    if (type == PLT_LIGHT_DISTANT) {
        // sample_cone (MathHelpers.slang:270-276) in the light's frame
        const float z = ux * (1.f - L.cosSubtendedAngle) + L.cosSubtendedAngle;
        const float r = sqrtf(1.f - z * z);
        float sp, cp;
        sincosf(k2Pi * uy, &sp, &cp);
        const f3 d = mk3(r * cp, r * sp, z);
        dir = normalize(mk3(L.xf[0] * d.x + L.xf[1] * d.y + L.xf[2] * d.z, L.xf[4] * d.x + L.xf[5] * d.y + L.xf[6] * d.z,
                            L.xf[8] * d.x + L.xf[9] * d.y + L.xf[10] * d.z));
        dist = kFltMax;
        const float solidAngle = k2Pi * (1.f - L.cosSubtendedAngle);
        sampleSpectrum<H>(P, L.spectrumId, wavelength, sg, importance, Li, wl);
        pdf = 1.f / solidAngle;
        return true;
    }
    // area lights: a point on the shape in object space, then finalizeAreaLightSample
    f3 lp, n;
    if (type == PLT_LIGHT_RECT) {
        lp = mk3(ux * 2.f - 1.f, uy * 2.f - 1.f, 0.f);
    } else if (type == PLT_LIGHT_DISC) {
        const float r = sqrtf(ux);
        float sp, cp;
        sincosf(k2Pi * uy, &sp, &cp);
        lp = mk3(r * cp, r * sp, 0.f);
    } else {
        float sp, cp;
        sincosf(k2Pi * uy, &sp, &cp);
        const float ct = 1.0f - 2.0f * ux;
        const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
        lp = mk3(st * cp, st * sp, ct);
    }
    const f3 posW = mk3(L.xf[0] * lp.x + L.xf[1] * lp.y + L.xf[2] * lp.z + L.xf[3], L.xf[4] * lp.x + L.xf[5] * lp.y + L.xf[6] * lp.z + L.xf[7],
                        L.xf[8] * lp.x + L.xf[9] * lp.y + L.xf[10] * lp.z + L.xf[11]);
    if (type == PLT_LIGHT_SPHERE)
        n = normalize(mk3(L.xfIT[0] * lp.x + L.xfIT[1] * lp.y + L.xfIT[2] * lp.z, L.xfIT[3] * lp.x + L.xfIT[4] * lp.y + L.xfIT[5] * lp.z,
                          L.xfIT[6] * lp.x + L.xfIT[7] * lp.y + L.xfIT[8] * lp.z));
    else
        n = mk3(L.nrm[0], L.nrm[1], L.nrm[2]);
    const f3 toLight = posW - p;
    const float distSqr = fmaxf(dot(toLight, toLight), 1e-9f);
    dist = sqrtf(distSqr);
    dir = toLight / dist;
    const float cosTheta = dot(n, -dir);
    if (cosTheta <= 0.f) return false;
    sampleSpectrum<H>(P, L.spectrumId, wavelength, sg, importance, Li, wl);
#pragma unroll
    for (int j = 0; j < H; ++j) Li[j] *= L.surfaceArea * cosTheta / distSqr;
    pdf = distSqr / (cosTheta * L.surfaceArea);
    return true;
}

// evalTrianglePdf x triangle-selection pdf (EmissiveLightSamplerHelpers.slang:120-151,
// EmissivePowerSampler.slang:81-122)
PLT_DI float emissivePdf(const PtParams& P, const PtScene& S, f3 posW, uint32_t light, f3 hitPos, f3 hitNormal) {
    if (light == kNoHit) return 0.f;
    // EmissiveUniformSampler.evalTriangleSelectionPdf (EmissiveUniformSampler.slang) or the power sampler's
    const float sel = (P.opt & plt::kPtUniformEmissive) ? (S.nActive > 0 ? 1.f / (float)S.nActive : 0.f)
                                                         : __ldg(P.lightFlux + light) * S.invWeightsSum;
    const f3 toLight = hitPos - posW;
    const float distSqr = dot(toLight, toLight);
    if (distSqr <= kFltMin) return 0.f;
    const f3 L = toLight / sqrtf(distSqr);
    const float cosTheta = dot(hitNormal, -L);
    if (cosTheta <= 0.f) return 0.f;
    const float denom = fmaxf(kFltMin, cosTheta * __ldg(P.lightArea + light));
    return sel * (distSqr / denom);
}

// A deferred forward replay (no manifold vertices): the beam as sourced and weighted at vertex p of
// path pid, to be replayed through vertex p (NEE on non-delta lobes: evalCurrent) and p-1 .. 0 and
// measured.  The replay draws no random numbers, so it can run after the solve kernel in any order.
template <int H> struct ReplayTask {
    PBeam<H> pb;
    uint32_t pid, p, evalCurrent;
};

// Hands a replay to the replay wavefront; false when the queue is full (the caller replays inline).
template <int H>
PLT_DI bool deferReplay(const PtParams& P, uint32_t pid, int p, bool evalCurrent, const PBeam<H>& pb) {
    const uint32_t slot = warpAggregatedAdd(P.replayCount, true);
    if (slot >= P.replayCap) return false;
    ReplayTask<H>* t = reinterpret_cast<ReplayTask<H>*>(static_cast<char*>(P.replayTasks) + (size_t)slot * plt::kReplayTaskBytes);
    t->pb = pb;
    t->pid = pid;
    t->p = (uint32_t)p;
    t->evalCurrent = evalCurrent ? 1u : 0u;
    return true;
}

// MNEE = false compiles the solve kernel without manifold sampling (the do_mnee = 0 pass): the
// occluder search and the task hand-off would otherwise enlarge the kernel for every option set.
// Resident CTAs of 128 threads per SM the solve kernel is compiled for: 16, the SM's 64 warps, at
// 32 registers (the rest of its state spills to local memory, which stays in L1).  Measured per
// 1024^2 frame with the walk kernel at 5 (three runs, each against its own baseline): 1 (228
// registers, 2 CTAs) 16.34 ms, 5 14.93, 7 14.06, 8 13.83; 8 14.18, 10 13.77, 12 13.54; 10 13.61,
// 12 13.72, 14 12.99, 16 12.98.  The kernel is latency-bound (traversal, scattered path records),
// and the extra warps hide more than the spills cost.
#ifndef PLT_SOLVE_MIN_BLOCKS
#define PLT_SOLVE_MIN_BLOCKS 16
#endif
template <int H, bool MNEE>
__global__ void __launch_bounds__(128, PLT_SOLVE_MIN_BLOCKS) ptSolveKernel(const PtParams P) {
    const float4* nodes = reinterpret_cast<const float4*>(P.nodes);
    const Ctx c{P.profiles, P.nProfiles, P.flags};
    const bool hwssMis = (P.opt & plt::kPtHwssMis) != 0;
    const bool doNee = (P.opt & plt::kPtDoNee) != 0, doMis = (P.opt & plt::kPtDoMis) != 0;
    const bool useEmissive = (P.opt & plt::kPtUseEmissive) != 0;
    const bool importance = (P.opt & plt::kPtImportanceEmit) != 0;
    const bool doMnee = MNEE && (P.opt & plt::kPtDoMnee) != 0;
    const bool useEnv = (P.opt & plt::kPtUseEnv) != 0;
    const bool useAnalytic = (P.opt & plt::kPtUseAnalytic) != 0;
    TraceCounters tc{0u, 0u, 0u, 0u};
    uint32_t evals = 0;
    MSData ms;
    for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < P.nWave; slot += gridDim.x * blockDim.x) {
        const uint32_t pid = (uint32_t)pltIdx(P.status, P.order ? P.order[pltIdx(P.status, slot, P.npix, kSiteQueue)] : slot, P.npix, kSitePath);
        const uint32_t gp = (uint32_t)pltIdx(P.status, P.pidBase + pid, P.nTotal, kSiteAccum);
        const PtScene& S = P.scenes[sceneOf(P, gp)];
        const int32_t root = (int32_t)S.root;
        const uint32_t local = gp - S.pixelBase;
        const uint32_t px = local % S.width, py = local / S.width;
        SampleGen sg, tilesg;
        const uint32_t frame = *P.frameDev;
        const bool tinySg = (P.opt & plt::kPtTinySg) != 0;
        sg.init(px, py, frame, tinySg);
        tilesg.init(px / P.tileSize, py / P.tileSize, frame << 2, tinySg);
        const float wavelength = 380.0f + sg.next1D() * (720.0f - 380.0f);
        f3 pathOrigin = camPos(S);
        // light-type selection probabilities (getLightTypeSelectionProbabilities,
        // LightSampling.slangh:40-55): the environment map, this scene's emissive geometry and the
        // analytic lights
        const bool hasEm = useEmissive && S.nActive > 0;   // Scene::useEmissiveLights: active lights present
        const float pSum = (useEnv ? 1.f : 0.f) + (hasEm ? 1.f : 0.f) + (useAnalytic ? 1.f : 0.f);
        const float invPSum = pSum > 0.f ? 1.f / pSum : 0.f;
        const float pEnv = useEnv ? invPSum : 0.f, pEm = hasEm ? invPSum : 0.f, pAn = useAnalytic ? invPSum : 0.f;
        float Lr = 0.f, Lg = 0.f, Lb = 0.f;
        DebugAcc dacc{0.f, 0.f, 0.f, 0.f};
        DebugAcc* dbg = P.debugView ? &dacc : nullptr;
        for (int p = 0; p <= (int)P.maxBounces; ++p) {
            const Bnc<H> bounce = readBounce<H>(P, pid, p);
            // wasNEEAvailable, pltpt_solve.rt.slang:204-210
            const bool didNEE = doNee && p > 0 &&
                                ((bounce.flags & kFlagLastDelta) == 0 || (doMnee && (bounce.flags >> 16) <= P.mneeMaxOccluders && p > 1));
            if (bounce.flags & kFlagMiss) {
                // onMiss, pltpt_solve.rt.slang:374-395: the environment map seen along the escaped
                // ray, a distant beam replayed through vertices p-1 .. 0
                if (useEnv && (doMis || !didNEE)) {
                    const f3 wo = bounce.wi;
                    const bool needMIS = doMis && didNEE;
                    const float lightPdf = pEnv * envEvalPdf(P.env, -wo);
                    const float mw = needMIS ? misWeight(bounce.lndp, lightPdf) : 1.f;
                    float Le[H], swl[H];
                    hwssWavelengths<H>(wavelength, swl);
                    const f3 rad = envEval(P.env, -wo);
#pragma unroll
                    for (int j = 0; j < H; ++j) Le[j] = mw * rgbToSpectrumAt(rad, swl[j]);
                    PBeam<H> pb;
                    sourceBeamDistant<H>(pb, wo, P.maxBeamOmega, Le, swl, P.maxBeamOmega);
                    if (!hwssMis && (bounce.flags & kFlagDispersive)) pb.comps = 1;
                    if (!(P.replayTasks && !dbg && deferReplay<H>(P, pid, p, false, pb)))
                        replayInline<H>(P, S, pid, p, bounce, pb, ms, 0, pathOrigin, false, c, hwssMis, Lr, Lg, Lb, evals, dbg);
                }
                break;
            }
            if (bounce.prim >= P.nTris) break;     // empty terminal record
            const VData V = vertexData(P, bounce.prim, bounce.b1, bounce.b2);
            const uint32_t mid = __ldg(P.triMat + bounce.prim);
            const uint2 props = __ldg(P.matProps + mid);
            const SD sd = prepareSD(V, props.x, bounce.wi);
            const DevMaterial* __restrict__ m = P.mats + mid;
            const uint32_t type = __ldg(&m->type);
            const uint32_t lobes = (props.x >> 8) & 0xFFu;
            if (dbg && p == 0) {
                // geometry views at the primary hit (pltpt_solve.rt.slang:449-456); the scene has no
                // texture coordinates, so sd.uv = 0
                dbgWrite(dbg, P.debugView, PLT_DEBUG_VIEW_NORMALS, sd.N);
                dbgWrite(dbg, P.debugView, PLT_DEBUG_VIEW_UVS, mk3(0.f, 0.f, 0.f));
            }
            // two beam sources per vertex: NEE (pltpt_solve.rt.slang:245-366) and emission
            // (evalEmissive, :152-200); each is replayed through vertices p (NEE: non-delta lobes)
            // and p-1 .. 0 (forwardUnwind, :48-79), then measured (:96-147).
            for (int src = 0; src < 2; ++src) {
                PBeam<H> pb;
                bool evalCurrent = false;
                int nMs = 0;            // manifold vertices to replay first (NEE with manifold walks)
                f3 msOrigin = pathOrigin;
                if (src == 0) {
                    if (!doNee) continue;
                    const bool allowMS = doMnee && p > 0 && (bounce.flags & kFlagLastDelta) == 0 && (props.x & plt::kPropMwReflective) != 0;
                    const bool sampleRefl = (lobes & 0x03u) != 0 || allowMS, sampleTrans = (lobes & 0x30u) != 0;
                    if (!sampleRefl && !sampleTrans) continue;
                    // generateLightSample (LightSampling.slangh:166-206): selectLightType (one
                    // draw), then the environment map's or the emissive power sampler's sample
                    SampleGen& selSg = (P.opt & plt::kPtPerTileSg) ? tilesg : sg;
                    float uType = selSg.next1D();
                    float selPdf;
                    int kind;   // 0 environment map, 1 emissive geometry, 2 analytic light
                    if (uType < pEnv) {
                        selPdf = pEnv;
                        kind = 0;
                    } else {
                        uType -= pEnv;
                        if (uType < pEm) {
                            selPdf = pEm;
                            kind = 1;
                        } else {
                            uType -= pEm;
                            if (!(uType < pAn)) continue;
                            selPdf = pAn;
                            kind = 2;
                        }
                    }
                    bool distant = kind == 0;
                    const bool misHere = doMis && kind != 2;   // no MIS for analytic lights (pltpt_solve.rt.slang:276)
                    const float invSel = 1.f / selPdf;
                    float Le[H], swl[H];
                    float tpdf;
                    bool anyPos = false;
                    f3 tposW, lorg, ldir;
                    float ldist, srcSize;
                    if (distant) {
                        // generateEnvMapSample (LightSampling.slangh:86-104, EnvMapSampler.slang:52-113)
                        const float e0 = sg.next1D();
                        const float e1 = sg.next1D();
                        float epdf;
                        ldir = envSampleDir(P.env, e0, e1, epdf);
                        hwssWavelengths<H>(wavelength, swl);
                        const f3 rad = envEval(P.env, ldir);
#pragma unroll
                        for (int j = 0; j < H; ++j) {
                            const float le = rgbToSpectrumAt(rad, swl[j]);
                            Le[j] = epdf > 0.f ? le / epdf : 0.f;
                            anyPos = anyPos || Le[j] > 0.f;
                            Le[j] *= invSel;
                        }
                        tpdf = epdf * selPdf;
                        lorg = newRayOriginToward(sd, ldir);
                        ldist = kFltMax;
                        tposW = lorg;
                        srcSize = P.maxBeamOmega;
                        sourceBeamDistant<H>(pb, -ldir, srcSize, Le, swl, P.maxBeamOmega);
                    } else if (kind == 2) {
                        // generateAnalyticLightSample (LightSampling.slangh:128-164): a light
                        // chosen uniformly, sampleLight, a distant or an area beam
                        const uint32_t nA = P.nALights;
                        const uint32_t li = min((uint32_t)(sg.next1D() * (float)nA), nA - 1);
                        const plt::AnalyticLightDev& AL = P.alights[li];
                        float apdf;
                        if (!sampleAnalytic<H>(P, AL, sd.posW, wavelength, sg, importance, ldir, ldist, Le, swl, apdf)) continue;
#pragma unroll
                        for (int j = 0; j < H; ++j) {
                            Le[j] *= (float)nA;
                            anyPos = anyPos || Le[j] > 0.f;
                            Le[j] *= invSel;
                        }
                        tpdf = (apdf / (float)nA) * selPdf;
                        lorg = newRayOriginToward(sd, ldir);
                        distant = AL.type == PLT_LIGHT_DIRECTIONAL || AL.type == PLT_LIGHT_DISTANT;
                        if (distant) {
                            // Omega = 4 pi (1 - cos^2) as the reference computes it
                            srcSize = 4.f * kPi * (1.f - AL.cosSubtendedAngle * AL.cosSubtendedAngle);
                            tposW = mk3(0.f, 0.f, 0.f);
                            sourceBeamDistant<H>(pb, -ldir, srcSize, Le, swl, P.maxBeamOmega);
                        } else {
                            srcSize = AL.surfaceArea;
                            tposW = mk3(AL.pos[0], AL.pos[1], AL.pos[2]);
                            sourceBeamArea<H>(pb, tposW, -ldir, srcSize, ldist, Le, swl, P.maxBeamOmega);
                        }
                    } else {
                        uint32_t ti;
                        float triSelPdf;
                        if (P.opt & plt::kPtUniformEmissive) {
                            // EmissiveUniformSampler.sampleLight: one draw over the active triangles
                            const float uLight = sg.next1D();
                            const uint32_t idx = min((uint32_t)(uLight * (float)S.nActive), S.nActive - 1);
                            ti = __ldg(P.lightActive + S.activeBase + idx);
                            triSelPdf = 1.f / (float)S.nActive;
                        } else {
                            const float uLight = sg.next1D();
                            ti = min((uint32_t)(uLight * (float)S.nLights), S.nLights - 1);
                            const uint2 a = __ldg(P.alias + S.lightBase + ti);
                            const float threshold = __half2float(__ushort_as_half((unsigned short)(a.x >> 16)));
                            const uint32_t selectAbove = ((a.x & 0xFFFFu) << 8u) | ((a.y >> 24u) & 0xFFu);
                            const uint32_t selectBelow = a.y & 0xFFFFFFu;
                            ti = S.lightBase + ((sg.next1D() >= threshold) ? selectAbove : selectBelow);
                            triSelPdf = __ldg(P.lightFlux + ti) * S.invWeightsSum;
                        }
                        const float u0 = sg.next1D(), u1 = sg.next1D();
                        const float su = sqrtf(u0);
                        const float bx = 1.f - su, by = u1 * su;
                        const float* LP = P.lightPos + 9 * ti;
                        tposW = ld3s(LP, 0) * (1.f - bx - by) + ld3s(LP, 1) * bx + ld3s(LP, 2) * by;
                        const f3 toL = tposW - sd.posW;
                        const float distSqr = fmaxf(kFltMin, dot(toL, toL));
                        const float tdist = sqrtf(distSqr);
                        const f3 tdir = toL / tdist;
                        const f3 tn = ld3s(P.lightNrm, ti);
                        const float cosTheta = dot(tn, -tdir);
                        if (cosTheta <= 0.f) continue;
                        sampleSpectrum<H>(P, __ldg(P.lightEmission + ti), wavelength, sg, importance, Le, swl);
                        const float epdf = (distSqr / fmaxf(kFltMin, cosTheta * __ldg(P.lightArea + ti))) * triSelPdf;
#pragma unroll
                        for (int j = 0; j < H; ++j) {
                            Le[j] *= whiteSpectrum(swl[j]);
                            Le[j] = epdf > 0.f ? Le[j] / epdf : 0.f;
                            anyPos = anyPos || Le[j] > 0.f;
                            Le[j] *= invSel;
                        }
                        tpdf = epdf * selPdf;
                        const f3 lightPos = computeRayOrigin(tposW, tn);
                        lorg = newRayOriginToward(sd, lightPos - sd.posW);
                        const f3 toLight = lightPos - lorg;
                        ldist = sqrtf(dot(toLight, toLight));
                        ldir = rnormalize(toLight);
                        srcSize = P.sourcingArea;
                        sourceBeamArea<H>(pb, tposW, -ldir, srcSize, ldist, Le, swl, P.maxBeamOmega);
                    }
                    const bool isRefl = dot(sd.faceN, ldir) * dot(sd.faceN, sd.V) > 0.f;
                    if (!(anyPos && tpdf > 1e-6f && !(!sampleRefl && isRefl) && !(!sampleTrans && !isRefl))) continue;
                    if (!hwssMis && (bounce.flags & kFlagDispersive)) pb.comps = 1;
                    const int maxMS = (int)P.maxBounces - p;
                    evalCurrent = true;
                    if (!doMnee || maxMS <= 0) {
                        ++tc.shadowRays;
                        const TraceResult vis =
                            traverse<true>(nodes, P.tris, lorg.x, lorg.y, lorg.z, ldir.x, ldir.y, ldir.z, 0.f, ldist, tc.nv, tc.tt, tc.overflow, root);
                        if (vis.prim != kNoHit) continue;
                        if (misHere) scaleBeam(pb, misWeight(tpdf, ptPdf(m, type, sd, ldir, pb.b.wl[0])));
                    } else {
                        // manifold sampling on NEE, pltpt_solve.rt.slang:293-353
                        const f3 lightDir = ldir;
                        ms.hitCount = 0;
                        ms.iterations = 0;
                        ms.wavelength = pb.b.wl[0];
                        ms.pdf = 1.f;
                        ms.dispersive = false;
                        const bool isRefl = dot(sd.N, lightDir) * dot(sd.N, sd.V) > 0.f;
                        const bool curMS = isRefl && allowMS;
                        if (curMS) {
                            if (!manifoldSampleVertex(P, bounce.prim, bounce.b1, bounce.b2, sd, mid, lightDir, sg, ms) ||
                                (ms.hits[0].lobe & kLobeReflection) == 0)
                                continue;
                        }
                        msOrigin = !curMS ? V.posW : pathOrigin;
                        const int occ = manifoldOccluders(P, root, lorg, ldir, ldist, maxMS, sg, ms, tc);
                        bool mneeOk = occ != kMsFail;
                        // without a debug view a sample with a negligible pdf is dropped before its walk
                        if (mneeOk && ms.pdf < 1e-6f && !dbg) continue;
                        if (occ == kMsWalk) {
                            // the walk and the rest of this sample draw no random numbers: hand them
                            // to the walk wavefront (inline when its queue is full)
                            const uint32_t slot = P.mneeTasks ? warpAggregatedAdd(P.mneeCount, true) : 0xFFFFFFFFu;
                            if (slot < P.mneeCap) {
                                MneeTask<H>* t = reinterpret_cast<MneeTask<H>*>(P.mneeTasks) + slot;
                                t->ms = ms;
                                t->tposW = tposW;
                                t->ldir = ldir;
                                t->msOrigin = msOrigin;
                                t->ldist = ldist;
                                t->tpdf = tpdf;
                                t->srcSize = srcSize;
#pragma unroll
                                for (int j = 0; j < H; ++j) { t->Le[j] = Le[j]; t->swl[j] = swl[j]; }
                                t->pid = pid;
                                t->p = (uint32_t)p;
                                t->curMS = (curMS ? 1u : 0u) | (distant ? 2u : 0u) | (misHere ? 0u : 4u);
                                continue;
                            }
                            mneeOk = manifoldWalk(P, root, msOrigin, tposW, ldir, distant, ms, tc);
                        }
                        if (dbg) {
                            // MNEE views (pltpt_solve.rt.slang:319-325)
                            dbgWrite(dbg, P.debugView, PLT_DEBUG_VIEW_MNEE_ITERATIONS,
                                     colourCode(kInferno, (float)ms.iterations / (float)P.mneeMaxIterations));
                            if (ms.hitCount > 0 && mneeOk)
                                dbgWrite(dbg, P.debugView, PLT_DEBUG_VIEW_MNEE_BOUNCES,
                                         ms.hitCount == 1 ? mk3(0.f, .3f, 1.f) : mk3(1.f, 0.f, 0.f));
                        }
                        if (!mneeOk || ms.pdf < 1e-6f) continue;
                        float misBsdfPdf = 0.f;
                        f3 lsDir = ldir;
                        if (ms.hitCount > 0) {
                            // (a distant light's beam already points along -woLastHitToLight)
                            if (!hwssMis && ms.dispersive) pb.comps = 1;
                            lsDir = ms.woLastHitToLight;
                            pb.b.r = -ms.woLastHitToLight;
                            pb.b.t = perp_stark(pb.b.r);
                            scaleBeam(pb, 1.f / ms.pdf);
                            nMs = ms.hitCount;
                            if (curMS) {
                                evalCurrent = false;
                                misBsdfPdf = bounce.lndp;
                            }
                        }
                        if (misHere) {
                            if (ms.hitCount == 0 || !curMS) misBsdfPdf = ptPdf(m, type, sd, lsDir, pb.b.wl[0]);
                            scaleBeam(pb, misWeight(tpdf, misBsdfPdf * ms.pdf));
                        }
                    }
                } else {
                    if (!(useEmissive && (props.x & plt::kPropEmissive) && (doMis || !didNEE))) continue;
                    const bool needMIS = doMis && didNEE;
                    const uint32_t light = __ldg(P.primToLight + bounce.prim);
                    const f3 hn = sd.frontFacing ? sd.faceN : -sd.faceN;
                    const float lightPdf = pEm * emissivePdf(P, S, pathOrigin, light, sd.posW, hn);
                    const float mw = needMIS ? misWeight(bounce.lndp, lightPdf) : 1.f;
                    float Le[H], swl[H];
                    sampleSpectrum<H>(P, props.y, wavelength, sg, importance, Le, swl);
                    bool anyPos = false;
#pragma unroll
                    for (int j = 0; j < H; ++j) {
                        Le[j] *= mw * whiteSpectrum(swl[j]);
                        anyPos = anyPos || Le[j] > 0.f;
                    }
                    if (!anyPos) continue;
                    const float dist = sqrtf(dot(pathOrigin - sd.posW, pathOrigin - sd.posW));
                    sourceBeamArea<H>(pb, sd.posW, bounce.wi, P.sourcingArea, dist, Le, swl, P.maxBeamOmega);
                    if (!hwssMis && (bounce.flags & kFlagDispersive)) pb.comps = 1;
                }
                if (!(nMs == 0 && P.replayTasks && !dbg && deferReplay<H>(P, pid, p, evalCurrent, pb)))
                    replayInline<H>(P, S, pid, p, bounce, pb, ms, nMs, msOrigin, evalCurrent, c, hwssMis, Lr, Lg, Lb, evals, dbg);
            }
            if ((bounce.flags & kFlagTerminated) || p == (int)P.maxBounces) break;
            pathOrigin = V.posW;
        }
        if (dbg) {
            // the output colour moves towards the mean debug colour by the view intensity
            // (pltpt_solve.rt.slang:470-475)
            const float t = P.debugIntensity;
            const f3 dm = dacc.n > 0.f ? mk3(dacc.r, dacc.g, dacc.b) / dacc.n : mk3(0.f, 0.f, 0.f);
            Lr = Lr + t * (dm.x - Lr);
            Lg = Lg + t * (dm.y - Lg);
            Lb = Lb + t * (dm.z - Lb);
        }
        P.accum[3 * (size_t)gp] += (double)Lr;
        P.accum[3 * (size_t)gp + 1] += (double)Lg;
        P.accum[3 * (size_t)gp + 2] += (double)Lb;
    }
    if (tc.overflow) atomicOr(P.status, plt::kStatusStackOverflow);
    unsigned long long s1 = tc.shadowRays, s2 = evals;
    for (int o = 16; o > 0; o >>= 1) {
        s1 += __shfl_down_sync(0xFFFFFFFFu, s1, o);
        s2 += __shfl_down_sync(0xFFFFFFFFu, s2, o);
    }
    if ((threadIdx.x & 31u) == 0) {
        if (s1) atomicAdd(P.stats + 1, s1);
        if (s2) atomicAdd(P.stats + 2, s2);
    }
    addTraversalBytes(P, tc.nv, tc.tt);
}


// The manifold-walk wavefront: one thread per deferred NEE sample (ptSolveKernel's MneeTask), dense
// in the walking lanes that the solve kernel's warps would otherwise run one or two at a time.
// Finishes the sample exactly as the solve kernel would (pltpt_solve.rt.slang:293-366: the walk,
// the beam's new direction, 1 / pdf, the MIS weight, the manifold replay and the measurement) and
// adds it to the pixel's accumulator.
// Resident CTAs per SM of the walk kernel: an early version measured 1 (128 registers) 16.05 ms per
// frame, 5 (96) 14.77 ms, 6 14.92 ms; the current one 4 (128 registers) 11.97 ms, 5 12.26 ms and 6
// 12.20 ms.
#ifndef PLT_MNEE_MIN_BLOCKS
#define PLT_MNEE_MIN_BLOCKS 4
#endif
template <int H>
__global__ void __launch_bounds__(128, PLT_MNEE_MIN_BLOCKS) ptMneeKernel(const PtParams P) {
    static_assert(sizeof(MneeTask<H>) <= plt::kMneeTaskBytes, "MneeTask stride");
    const uint32_t count = min(*((volatile uint32_t*)P.mneeCount), P.mneeCap);
    const Ctx c{P.profiles, P.nProfiles, P.flags};
    const bool hwssMis = (P.opt & plt::kPtHwssMis) != 0;
    const bool doMis = (P.opt & plt::kPtDoMis) != 0;
    TraceCounters tc{0u, 0u, 0u, 0u};
    uint32_t evals = 0;
    const MneeTask<H>* tasks = reinterpret_cast<const MneeTask<H>*>(P.mneeTasks);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const MneeTask<H>& t = tasks[pltIdx(P.status, P.mneeOrder ? P.mneeOrder[pltIdx(P.status, i, P.mneeCap, kSiteTask)] : i, P.mneeCap, kSiteTask)];
        MSData ms = t.ms;
        const uint32_t pid = t.pid;
        const int p = (int)t.p;
        const bool curMS = (t.curMS & 1u) != 0;
        const bool distant = (t.curMS & 2u) != 0;
        const bool misHere = doMis && (t.curMS & 4u) == 0;
        const f3 msOrigin = t.msOrigin;
        const uint32_t gp = (uint32_t)pltIdx(P.status, P.pidBase + pid, P.nTotal, kSiteAccum);
        const PtScene& S = P.scenes[sceneOf(P, gp)];
        if (!manifoldWalk(P, (int32_t)S.root, msOrigin, t.tposW, t.ldir, distant, ms, tc)) continue;
        const Bnc<H> bounce = readBounce<H>(P, pid, p);
        const VData V = vertexData(P, bounce.prim, bounce.b1, bounce.b2);
        const uint32_t mid = __ldg(P.triMat + bounce.prim);
        const SD sd = prepareSD(V, __ldg(P.matProps + mid).x, bounce.wi);
        const DevMaterial* __restrict__ m = P.mats + mid;
        const uint32_t type = __ldg(&m->type);
        float Le[H], swl[H];
#pragma unroll
        for (int j = 0; j < H; ++j) { Le[j] = t.Le[j]; swl[j] = t.swl[j]; }
        PBeam<H> pb;
        if (distant) sourceBeamDistant<H>(pb, -t.ldir, t.srcSize, Le, swl, P.maxBeamOmega);
        else sourceBeamArea<H>(pb, t.tposW, -t.ldir, t.srcSize, t.ldist, Le, swl, P.maxBeamOmega);
        if (!hwssMis && (bounce.flags & kFlagDispersive)) pb.comps = 1;
        bool evalCurrent = true;
        float misBsdfPdf = 0.f;
        if (!hwssMis && ms.dispersive) pb.comps = 1;
        const f3 lsDir = ms.woLastHitToLight;
        pb.b.r = -ms.woLastHitToLight;
        pb.b.t = perp_stark(pb.b.r);
        scaleBeam(pb, 1.f / ms.pdf);
        const int nMs = ms.hitCount;
        if (curMS) {
            evalCurrent = false;
            misBsdfPdf = bounce.lndp;
        }
        if (misHere) {
            if (!curMS) misBsdfPdf = ptPdf(m, type, sd, lsDir, pb.b.wl[0]);
            scaleBeam(pb, misWeight(t.tpdf, misBsdfPdf * ms.pdf));
        }
        float Lr = 0.f, Lg = 0.f, Lb = 0.f;
        replayMeasure<H>(P, S, pid, p, bounce, pb, ms, nMs, msOrigin, evalCurrent, c, hwssMis, Lr, Lg, Lb, evals);
        if (Lr != 0.f || Lg != 0.f || Lb != 0.f) {
            atomicAdd(P.accum + 3 * (size_t)gp, (double)Lr);
            atomicAdd(P.accum + 3 * (size_t)gp + 1, (double)Lg);
            atomicAdd(P.accum + 3 * (size_t)gp + 2, (double)Lb);
        }
    }
    if (tc.overflow) atomicOr(P.status, plt::kStatusStackOverflow);
    unsigned long long s1 = tc.shadowRays, s2 = evals;
    for (int o = 16; o > 0; o >>= 1) {
        s1 += __shfl_down_sync(0xFFFFFFFFu, s1, o);
        s2 += __shfl_down_sync(0xFFFFFFFFu, s2, o);
    }
    if ((threadIdx.x & 31u) == 0) {
        if (s1) atomicAdd(P.stats + 1, s1);
        if (s2) atomicAdd(P.stats + 2, s2);
    }
    addTraversalBytes(P, tc.nv, tc.tt);
}

// The walk wavefront's order: tasks counting-sorted by (occluder count, material group of the first
// occluder), so a warp's lanes run Newton walks of the same chain length over the same material
// code.  Count pass, then a scatter pass in which every block reserves its share of each key's
// slots after the exclusive prefix of the counts.
template <int H> PLT_DI uint32_t mneeKey(const PtParams& P, const MneeTask<H>& t) {
    const uint32_t hc = (uint32_t)min(max(t.ms.hitCount, 1), 4) - 1u;
    const uint32_t prim = t.ms.hits[0].prim;
    const uint32_t ty = prim < P.nTris ? __ldg(&P.mats[__ldg(P.triMat + prim)].type) : 0u;
    const uint32_t g = (ty == kMatDielectric || ty == kMatThin) ? 0u : (ty == kMatMultilayer) ? 1u
                     : (ty == kMatGratedConductor || ty == kMatGratedOpaque) ? 2u : 3u;
    return hc * 4u + g;
}
template <int H>
__global__ void __launch_bounds__(256) ptMneeCountKernel(const PtParams P) {
    __shared__ uint32_t h[16];
    if (threadIdx.x < 16) h[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t count = min(*((volatile uint32_t*)P.mneeCount), P.mneeCap);
    const MneeTask<H>* tasks = reinterpret_cast<const MneeTask<H>*>(P.mneeTasks);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        atomicAdd(&h[mneeKey<H>(P, tasks[i])], 1u);
    __syncthreads();
    if (threadIdx.x < 16 && h[threadIdx.x]) atomicAdd(P.mneeSort + threadIdx.x, h[threadIdx.x]);
}
template <int H>
__global__ void __launch_bounds__(256) ptMneeScatterKernel(const PtParams P) {
    __shared__ uint32_t h[16], base[16];
    const uint32_t count = min(*((volatile uint32_t*)P.mneeCount), P.mneeCap);
    const uint32_t per = (count + gridDim.x - 1) / gridDim.x;
    const uint32_t begin = min(blockIdx.x * per, count), end = min(begin + per, count);
    const MneeTask<H>* tasks = reinterpret_cast<const MneeTask<H>*>(P.mneeTasks);
    if (threadIdx.x < 16) h[threadIdx.x] = 0;
    __syncthreads();
    for (uint32_t i = begin + threadIdx.x; i < end; i += blockDim.x) atomicAdd(&h[mneeKey<H>(P, tasks[i])], 1u);
    __syncthreads();
    if (threadIdx.x < 16) {
        uint32_t prefix = 0;
        for (uint32_t k = 0; k < threadIdx.x; ++k) prefix += P.mneeSort[k];
        base[threadIdx.x] = h[threadIdx.x] ? prefix + atomicAdd(P.mneeSort + 16 + threadIdx.x, h[threadIdx.x]) : 0u;
        h[threadIdx.x] = 0;
    }
    __syncthreads();
    for (uint32_t i = begin + threadIdx.x; i < end; i += blockDim.x) {
        const uint32_t k = mneeKey<H>(P, tasks[i]);
        P.mneeOrder[base[k] + atomicAdd(&h[k], 1u)] = i;
    }
}
// The replay wavefront: the solve kernel's deferred replays counting-sorted by (material type of
// the first vertex to evaluate, vertices to evaluate), so a warp's lanes evaluate the same material
// code over paths of the same length (the material-sorted queue of the forward unwind,
// pltpt_solve.rt.slang:48-79), then replayed one thread each and added to the pixel's accumulator.
// The replay kernel's warps take 32 consecutive tasks of that order at a time from one counter, so
// the warps resident on an SM at any moment work on neighbouring keys: one or two materials' code.
template <int H> PLT_DI uint32_t replayKey(const PtParams& P, const ReplayTask<H>& t) {
    const uint32_t nEval = t.p + t.evalCurrent;
    const int first = t.evalCurrent ? (int)t.p : (int)t.p - 1;
    uint32_t ty = 0;
    if (first >= 0) {
        const uint32_t prim = P.bPrim[(size_t)first * P.npix + t.pid];
        if (prim < P.nTris) ty = min(__ldg(&P.mats[__ldg(P.triMat + prim)].type), 15u);
    }
    return ty * 16u + min(nEval, 15u);
}
template <int H> PLT_DI const ReplayTask<H>& replayTask(const PtParams& P, uint32_t i) {
    return *reinterpret_cast<const ReplayTask<H>*>(static_cast<const char*>(P.replayTasks) + (size_t)i * plt::kReplayTaskBytes);
}
template <int H>
__global__ void __launch_bounds__(256) ptReplayCountKernel(const PtParams P) {
    __shared__ uint32_t h[plt::kReplayKeys];
    for (uint32_t b = threadIdx.x; b < plt::kReplayKeys; b += blockDim.x) h[b] = 0;
    __syncthreads();
    const uint32_t count = min(*((volatile uint32_t*)P.replayCount), P.replayCap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        atomicAdd(&h[replayKey<H>(P, replayTask<H>(P, i))], 1u);
    __syncthreads();
    for (uint32_t b = threadIdx.x; b < plt::kReplayKeys; b += blockDim.x)
        if (h[b]) atomicAdd(P.replaySort + b, h[b]);
}
template <int H>
__global__ void __launch_bounds__(256) ptReplayScatterKernel(const PtParams P) {
    __shared__ uint32_t h[plt::kReplayKeys], base[plt::kReplayKeys];
    const uint32_t count = min(*((volatile uint32_t*)P.replayCount), P.replayCap);
    const uint32_t per = (count + gridDim.x - 1) / gridDim.x;
    const uint32_t begin = min(blockIdx.x * per, count), end = min(begin + per, count);
    for (uint32_t b = threadIdx.x; b < plt::kReplayKeys; b += blockDim.x) h[b] = 0;
    __syncthreads();
    for (uint32_t i = begin + threadIdx.x; i < end; i += blockDim.x) atomicAdd(&h[replayKey<H>(P, replayTask<H>(P, i))], 1u);
    __syncthreads();
    // each key's first slot: the exclusive prefix of the key counts (warp scan over 8 keys per lane)
    if (threadIdx.x < 32) {
        constexpr uint32_t per8 = plt::kReplayKeys / 32;
        uint32_t s = 0;
        for (uint32_t j = 0; j < per8; ++j) s += P.replaySort[threadIdx.x * per8 + j];
        uint32_t incl = s;
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t v = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if ((int)threadIdx.x >= d) incl += v;
        }
        uint32_t run = incl - s;
        for (uint32_t j = 0; j < per8; ++j) {
            const uint32_t b = threadIdx.x * per8 + j;
            base[b] = h[b] ? run + atomicAdd(P.replaySort + plt::kReplayKeys + b, h[b]) : 0u;
            run += P.replaySort[b];
            h[b] = 0;
        }
    }
    __syncthreads();
    for (uint32_t i = begin + threadIdx.x; i < end; i += blockDim.x) {
        const uint32_t k = replayKey<H>(P, replayTask<H>(P, i));
        P.replayOrder[base[k] + atomicAdd(&h[k], 1u)] = i;
    }
}
// The replay kernel: each CTA takes 128 consecutive tasks of the sorted order (one counter), stages
// them in shared memory and replays them vertex by vertex.  Before each vertex the CTA counting-sorts
// its tasks by the material type of the vertex they evaluate next and thread t replays the task at
// sorted position t, so a warp's lanes run one material's eval code at every vertex, not only at the
// first (a task's later vertices are of any material).  Then each thread measures its own task.  A
// task's arithmetic is that of replayMeasure, vertex for vertex.
constexpr uint32_t kReplayCtaTasks = 128;
#ifndef PLT_REPLAY_MIN_BLOCKS
#define PLT_REPLAY_MIN_BLOCKS 1
#endif
template <int H>
__global__ void __launch_bounds__(kReplayCtaTasks, PLT_REPLAY_MIN_BLOCKS) ptReplayKernel(const PtParams P) {
    static_assert(sizeof(ReplayTask<H>) <= plt::kReplayTaskBytes, "ReplayTask stride");
    __shared__ __align__(16) unsigned char stBytes[kReplayCtaTasks * sizeof(ReplayTask<H>)];
    __shared__ uint32_t hist[17], taskAt[kReplayCtaTasks], chunk;
    ReplayTask<H>* st = reinterpret_cast<ReplayTask<H>*>(stBytes);
    const uint32_t count = min(*((volatile uint32_t*)P.replayCount), P.replayCap);
    const Ctx c{P.profiles, P.nProfiles, P.flags};
    const bool hwssMis = (P.opt & plt::kPtHwssMis) != 0;
    const uint32_t n = P.npix;
    const uint32_t t = threadIdx.x;
    uint32_t evals = 0;
    uint32_t* next = P.replaySort + 2 * plt::kReplayKeys;   // the CTAs' work counter
    for (;;) {
        if (t == 0) chunk = atomicAdd(next, kReplayCtaTasks);
        __syncthreads();
        const uint32_t c0 = chunk;
        if (c0 >= count) break;
        const uint32_t nHere = min(kReplayCtaTasks, count - c0);
        if (t < nHere) st[t] = replayTask<H>(P, (uint32_t)pltIdx(P.status, P.replayOrder[pltIdx(P.status, c0 + t, P.replayCap, kSiteTask)], P.replayCap, kSiteTask));
        __syncthreads();
        const uint32_t pid = t < nHere ? st[t].pid : 0u;
        const int p = t < nHere ? (int)st[t].p : 0;
        const uint32_t ec = t < nHere ? st[t].evalCurrent : 0u;
        const int total = t < nHere ? p + (int)ec : 0;
        for (int r = 0;; ++r) {
            // this thread's task: its vertex r (the current one first when it is evaluated, then
            // p-1 .. 0) and the material type there; 16 once the task has no vertex r
            uint32_t key = 16u;
            if (r < total) {
                const int q = (ec && r == 0) ? p : p - 1 - (r - (int)ec);
                const uint32_t prim = P.bPrim[(size_t)q * n + pid];
                key = prim < P.nTris ? min(__ldg(&P.mats[__ldg(P.triMat + prim)].type), 15u) : 0u;
            }
            if (t < 17) hist[t] = 0u;
            __syncthreads();
            const uint32_t rank = key < 16u ? atomicAdd(&hist[key], 1u) : 0u;
            __syncthreads();
            if (t == 0) {
                uint32_t run = 0;
                for (int k = 0; k < 16; ++k) {
                    const uint32_t h = hist[k];
                    hist[k] = run;
                    run += h;
                }
                hist[16] = run;
            }
            __syncthreads();
            const uint32_t active = hist[16];
            if (active == 0u) break;
            if (key < 16u) taskAt[hist[key] + rank] = t;
            __syncthreads();
            if (t < active) {
                ReplayTask<H>& T = st[taskAt[t]];
                const int tp = (int)T.p;
                const bool cur = T.evalCurrent && r == 0;
                const int q = cur ? tp : tp - 1 - (r - (int)T.evalCurrent);
                const Bnc<H> bq = readBounce<H>(P, T.pid, q);
                PBeam<H> pb = T.pb;
                replayVertex<H>(P, bq.prim, bq.b1, bq.b2, bq.wi, cur ? kLobeNonDelta : bq.lobe, false, mk3(0.f, 0.f, 0.f), pb, c, hwssMis, evals);
                T.pb = pb;
            }
            __syncthreads();
        }
        if (t < nHere) {
            const uint32_t gp = (uint32_t)pltIdx(P.status, P.pidBase + pid, P.nTotal, kSiteAccum);
            const PtScene& S = P.scenes[sceneOf(P, gp)];
            const Bnc<H> bounce = readBounce<H>(P, pid, p);
            PBeam<H> pb = st[t].pb;
            float Lr = 0.f, Lg = 0.f, Lb = 0.f;
            replayFinish<H>(P, S, p, bounce, pb, hwssMis, Lr, Lg, Lb, nullptr);
            if (Lr != 0.f || Lg != 0.f || Lb != 0.f) {
                atomicAdd(P.accum + 3 * (size_t)gp, (double)Lr);
                atomicAdd(P.accum + 3 * (size_t)gp + 1, (double)Lg);
                atomicAdd(P.accum + 3 * (size_t)gp + 2, (double)Lb);
            }
        }
        __syncthreads();   // the staged tasks and `chunk` are read before the next chunk replaces them
    }
    unsigned long long s2 = evals;
    for (int o = 16; o > 0; o >>= 1) s2 += __shfl_down_sync(0xFFFFFFFFu, s2, o);
    if ((threadIdx.x & 31u) == 0 && s2) atomicAdd(P.stats + 2, s2);
}

template <int H>
cudaError_t launchSolve(const PtParams& p, const plt::PtLaunch& L, int numSMs, cudaStream_t stream) {
    static int bps[2] = {-1, -1};
    const bool mnee = (p.opt & plt::kPtDoMnee) != 0;
    if (bps[mnee] < 0) {
        int b = 0;
        if (mnee) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ptSolveKernel<H, true>, 128, 0);
        else cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ptSolveKernel<H, false>, 128, 0);
        bps[mnee] = b > 0 ? b : 1;
    }
    uint32_t grid = (uint32_t)numSMs * (L.solveBlocksPerSM ? min((uint32_t)bps[mnee], L.solveBlocksPerSM) : (uint32_t)bps[mnee]);
    const uint32_t need = (p.nWave + 127) / 128;
    if (grid > need) grid = need;
    if (mnee) ptSolveKernel<H, true><<<grid, 128, 0, stream>>>(p);
    else ptSolveKernel<H, false><<<grid, 128, 0, stream>>>(p);
    if (mnee && p.mneeTasks) {
        const plt::NvtxRange r("pt_walks");
        static int bpsW = -1;
        if (bpsW < 0) {
            int b = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ptMneeKernel<H>, 128, 0);
            bpsW = b > 0 ? b : 1;
        }
        const uint32_t gw = (uint32_t)numSMs * (L.walkBlocksPerSM ? min((uint32_t)bpsW, L.walkBlocksPerSM) : (uint32_t)bpsW);
        if (p.mneeOrder && p.mneeSort) {
            ptMneeCountKernel<H><<<numSMs, 256, 0, stream>>>(p);
            ptMneeScatterKernel<H><<<numSMs, 256, 0, stream>>>(p);
        }
        ptMneeKernel<H><<<gw, 128, 0, stream>>>(p);
    }
    if (p.replayTasks) {
        const plt::NvtxRange r("pt_replays");
        static int bpsR = -1;
        if (bpsR < 0) {
            int b = 0;
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, ptReplayKernel<H>, kReplayCtaTasks, 0);
            bpsR = b > 0 ? b : 1;
        }
        ptReplayCountKernel<H><<<numSMs, 256, 0, stream>>>(p);
        ptReplayScatterKernel<H><<<numSMs, 256, 0, stream>>>(p);
        ptReplayKernel<H><<<(uint32_t)numSMs * (uint32_t)bpsR, kReplayCtaTasks, 0, stream>>>(p);
    }
    return cudaGetLastError();
}

// per-H solve launchers, one translation unit each (plt_pt_h{1,2,3,4}.cu)
template <int H> cudaError_t launchSolveH(const PtParams& p, const plt::PtLaunch& L, int numSMs, cudaStream_t stream);

}  // namespace pltdev
