// ORACLE -- test infrastructure only.  CPU restatement of the PLTPT render pass (sample pass,
// solve pass, light sampling, forward beam replay, measurement) of ssteinberg/PLTFalcor, used to
// check plt_render.  FP32, brute-force ray casting with the reference's watertight test, one path
// per pixel per frame.  Citations are to Source/RenderPasses/PLTPT/* and Source/Falcor/* in the
// reference; every function follows the cited lines.  The scene has identity instance transforms
// and no textures (materials read their constants), no environment map and no analytic lights, so
// the light-type selection always picks emissive geometry (LightSampling.slangh:40-90).
#include "plt_oracle.hpp"
#include "plt_oracle_bsdf.hpp"
#include "plt_oracle_env.hpp"
#include "plt_oracle_geom.hpp"
#include "plt_oracle_mlp.hpp"

#include <algorithm>
#include <array>
#include <cfloat>
#include <memory>
#include <random>
#include <type_traits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using namespace plt_oracle;

namespace {

using F3 = V3<float>;
inline F3 f3(const float* p) { return {p[0], p[1], p[2]}; }
inline void put(F3 v, float* p) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t FLAG_LAST_DELTA = 0x1u, FLAG_DISPERSIVE = 0x2u, FLAG_ONLY_DELTA = 0x4u, FLAG_MISS = 0x10u,
                   FLAG_TERMINATED = 0x20u;
// a vertex where the learned proposal was a sampling technique (no counterpart in the reference)
constexpr uint32_t FLAG_LEARNED = 0x40u;
constexpr float kQcutoffForMS = .15f;               // IMaterialInstance.slang:44
constexpr uint32_t PROP_EMISSIVE = 0x1u, PROP_TRANSMISSIVE = 0x2u, PROP_MW_REFLECTIVE = 0x4u, PROP_MW_TRANSMISSIVE = 0x8u;

// Bounce record (Path.slang:113-142): the hit, the oct-encoded incident direction, sampled lobe,
// flags, path contribution and last non-delta pdf.
struct Bounce {
    uint32_t prim = kNone;
    float b1 = 0.f, b2 = 0.f;
    float ewi[2] = {0.f, 0.f};
    uint32_t lobe = 0, flags = 0;
    float pathContribution = 0.f, lastNonDeltaPdf = 0.f;
    F3 wi() const { float n[3]; geom::octToNdirEqualArea(ewi, n); return f3(n); }
};

struct Scene {
    uint32_t nv = 0, nt = 0;
    const float* pos = nullptr;
    const float* nrm = nullptr;
    const float* tan = nullptr;
    const uint32_t* idx = nullptr;
    const uint32_t* triMat = nullptr;
    const uint32_t* triInst = nullptr;   // geometry instance of each triangle (MNEE re-projection), or null = 0
    std::vector<Material<float>> mats;
    std::vector<uint32_t> matFlags;
    SceneTables tables;
    std::vector<float> triVerts;       // [nt][9]
    geom::OracleBvh bvh;
    // light collection (LightCollection.cpp, EmissivePowerSampler.cpp)
    std::vector<uint32_t> lightTri;    // light triangle -> primitive
    std::vector<uint32_t> primToLight; // primitive -> light triangle or kNone
    std::vector<float> lightPos;       // [nl][9]
    std::vector<float> lightNormal;    // [nl][3] (2x16 snorm round trip)
    std::vector<float> lightArea, lightFlux;
    std::vector<uint32_t> alias;       // [nl][2]
    float invWeightsSum = 0.f;
    // learned proposal: network (bf16-rounded) and per-material (roughness, pitch, class, enabled)
    std::unique_ptr<plt_oracle_mlp::Net> net;
    std::vector<float> matFeat;        // [nmat][4]
    // environment light (EnvMap + EnvMapSampler), when present
    plt_oracle_env::EnvMap env;
    // analytic lights (LightData) with the inverse-transpose of each transform's 3x3 part
    std::vector<plt_analytic_light> alights;
    std::vector<std::array<float, 9>> alightsIT;
};

struct Options {
    uint32_t maxBounces, tileSize, hwss;
    bool hwssMis, useDirect, useEmissive, doNee, doMis, doRR, perTileSg, importanceSampleEmitters;
    float sourcingArea, maxBeamOmega;
    bool doMnee;
    uint32_t mneeMaxOccluders, mneeMaxIterations;
    float mneeThreshold;
    bool learned = false;
    float learnedProb = 0.5f;
    bool useEnv = false;
    bool useAnalytic = false;
    bool uniformEmissive = false;   // emissiveSampler = Uniform (else Power)
    bool alphaMask = true;          // alphaMasking
    bool tinySg = false;            // sampleGenerator = TinyUniform (else Uniform)
    uint32_t debugView = 0;         // DebugViewType
    float debugIntensity = 1.f;
};

// ---- debug views: writeDebugOutput and the colour maps of pltpt_debug.slangh / ColourCoding.slang
#include "../pltfalcor_gb300/csrc/plt_colour_maps.h"

F3 colourCode(const float (*t)[3], float val) {
    val *= 256.f;
    if (!std::isfinite(val)) return {NAN, 0.f, 0.f};
    const int l = std::clamp((int)val, 0, 255), h = std::clamp((int)(val + 1.f), 0, 255);
    const float fr = val - std::floor(val);
    const F3 a = {t[l][0], t[l][1], t[l][2]}, b = {t[h][0], t[h][1], t[h][2]};
    return a + (b - a) * fr;
}

// ---------------------------------------------------------------------------------------------
// Light collection and the power sampler's alias table
// ---------------------------------------------------------------------------------------------
// Emissive triangles are those of materials with an emission profile (PLTDiffuse, BasicMaterialData
// .isEmissive(), BasicMaterialData.slang:138), in primitive order.  Face normal and area as
// computeFaceNormalAndAreaW (Scene.slang:482-497); flux = luminance(profile rgb) * area * pi
// (FinalizeIntegration.cs.slang:60-110).
void buildLights(Scene& s) {
    s.primToLight.assign(s.nt, kNone);
    for (uint32_t t = 0; t < s.nt; ++t) {
        const uint32_t m = s.triMat[t];
        if (m >= s.mats.size()) continue;
        if (s.mats[m].type != PLT_MATERIAL_DIFFUSE || s.mats[m].emission == PLT_NO_SPECTRAL_PROFILE) continue;
        s.primToLight[t] = (uint32_t)s.lightTri.size();
        s.lightTri.push_back(t);
    }
    const uint32_t nl = (uint32_t)s.lightTri.size();
    s.lightPos.resize(9 * (size_t)nl);
    s.lightNormal.resize(3 * (size_t)nl);
    s.lightArea.resize(nl);
    s.lightFlux.resize(nl);
    for (uint32_t l = 0; l < nl; ++l) {
        const uint32_t t = s.lightTri[l];
        F3 p[3];
        for (int k = 0; k < 3; ++k) {
            p[k] = f3(s.pos + 3 * (size_t)s.idx[3 * (size_t)t + k]);
            put(p[k], &s.lightPos[9 * (size_t)l + 3 * k]);
        }
        const F3 N = cross(p[1] - p[0], p[2] - p[0]);
        const float area = 0.5f * length(N);
        const F3 n = normalize(N);
        const float nn[3] = {n.x, n.y, n.z};
        geom::quantizeNormal2x16(nn, &s.lightNormal[3 * (size_t)l]);
        s.lightArea[l] = area;
        const uint32_t em = s.mats[s.triMat[t]].emission;
        float rgb[3] = {0.f, 0.f, 0.f};
        if (em < s.tables.count) for (int c = 0; c < 3; ++c) rgb[c] = std::max(0.f, s.tables.profiles[em].rgb[c]);
        const float lum = rgb[0] * 0.2126f + rgb[1] * 0.7152f + rgb[2] * 0.0722f;
        s.lightFlux[l] = lum * area * (float)K_PI;
    }
    // Alias table, EmissivePowerSampler.cpp:86-175: scaled weights, sorted small to large (stable
    // sort here: the reference's std::sort leaves the order of equal weights unspecified), paired
    // head/tail, entries shuffled with a default-seeded mt19937, thresholds stored as binary16.
    const uint32_t N = nl;
    s.alias.assign(2 * (size_t)N, 0u);
    if (N == 0) { s.invWeightsSum = 0.f; return; }
    std::vector<float> w(s.lightFlux);
    double sum = 0.0;
    for (float f : w) sum += f;
    for (float& f : w) f *= N / float(sum);
    std::vector<uint32_t> perm(N);
    for (uint32_t i = 0; i < N; ++i) perm[i] = i;
    std::stable_sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) { return w[a] < w[b]; });
    std::vector<float> thr(N, 0.f);
    std::vector<uint32_t> red(N, 0u);
    uint32_t head = 0, tail = N - 1;
    while (head != tail) {
        const uint32_t i = perm[head], j = perm[tail];
        thr[i] = w[i];
        red[i] = j;
        w[j] -= 1.0f - w[i];
        if (head == tail - 1) {
            thr[j] = 1.0f;
            red[j] = j;
            break;
        } else if (w[j] < 1.0f) {
            std::swap(perm[head], perm[tail]);
            tail--;
        } else {
            head++;
        }
    }
    for (uint32_t i = 0; i < N; ++i) perm[i] = i;
    std::mt19937 rng;
    for (uint32_t i = 0; i < N; ++i) {
        const uint32_t dst = i + ((uint32_t)rng() % (N - i));
        std::swap(thr[i], thr[dst]);
        std::swap(red[i], red[dst]);
        std::swap(perm[i], perm[dst]);
    }
    for (uint32_t i = 0; i < N; ++i) {
        const uint32_t prob = (uint32_t)geom::floatToHalfRne(thr[i]) << 16u;
        const uint32_t lx = red[i] & 0xFFFFFFu, ly = perm[i] & 0xFFFFFFu;
        s.alias[2 * (size_t)i] = prob | ((lx >> 8u) & 0xFFFFu);
        s.alias[2 * (size_t)i + 1] = ((lx & 0xFFu) << 24u) | ly;
    }
    s.invWeightsSum = 1.0f / float(sum);
}

// ---------------------------------------------------------------------------------------------
// Vertex and shading data
// ---------------------------------------------------------------------------------------------
struct VertexData {
    F3 posW, normalW, faceNormalW;
    float tangentW[4];
};
// computeVertexData, Scene.slang:530-567 (identity world matrix, front face CCW)
VertexData vertexData(const Scene& s, uint32_t prim, float b1, float b2) {
    const float w[3] = {1.f - b1 - b2, b1, b2};
    VertexData v;
    const uint32_t* I = s.idx + 3 * (size_t)prim;
    F3 p[3];
    for (int k = 0; k < 3; ++k) p[k] = f3(s.pos + 3 * (size_t)I[k]);
    v.posW = p[0] * w[0];
    v.posW = v.posW + p[1] * w[1];
    v.posW = v.posW + p[2] * w[2];
    F3 n = f3(s.nrm + 3 * (size_t)I[0]) * w[0];
    n = n + f3(s.nrm + 3 * (size_t)I[1]) * w[1];
    n = n + f3(s.nrm + 3 * (size_t)I[2]) * w[2];
    v.normalW = normalize(n);
    v.faceNormalW = normalize(cross(p[1] - p[0], p[2] - p[0]));
    if (s.tan) {
        float t[4] = {0.f, 0.f, 0.f, 0.f};
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 4; ++c) t[c] = (k == 0) ? s.tan[4 * (size_t)I[0] + c] * w[0] : t[c] + s.tan[4 * (size_t)I[k] + c] * w[k];
        const F3 tx = normalize(F3{t[0], t[1], t[2]});
        v.tangentW[0] = tx.x; v.tangentW[1] = tx.y; v.tangentW[2] = tx.z;
        v.tangentW[3] = geom::hsign(t[3]);
    } else {
        v.tangentW[0] = v.tangentW[1] = v.tangentW[2] = v.tangentW[3] = 0.f;
    }
    return v;
}

struct ShadingData {
    F3 posW, V, N, T, B, faceN;
    bool frontFacing = true;
    uint32_t materialID = 0;
    float opacity = 1.f;
    F3 toLocal(F3 v) const { return {dot(v, T), dot(v, B), dot(v, N)}; }
    F3 fromLocal(F3 v) const { return T * v.x + B * v.y + N * v.z; }
    // ShadingData.computeNewRayOrigin, ShadingData.slang:77-80
    F3 newRayOrigin(bool viewside = true) const {
        const F3 n = (frontFacing == viewside) ? faceN : -faceN;
        const float p[3] = {posW.x, posW.y, posW.z}, nn[3] = {n.x, n.y, n.z};
        float o[3];
        geom::computeRayOrigin(p, nn, o);
        return f3(o);
    }
};
// computeNewRayOrigin(sd, dir), ShadowRays.slangh:50-52
F3 newRayOriginToward(const ShadingData& sd, F3 dir) {
    const F3 n = dot(sd.faceN, dir) >= 0.f ? sd.faceN : -sd.faceN;
    const float p[3] = {sd.posW.x, sd.posW.y, sd.posW.z}, nn[3] = {n.x, n.y, n.z};
    float o[3];
    geom::computeRayOrigin(p, nn, o);
    return f3(o);
}

// MaterialHeader double-sided flag, forced on for specular or diffuse transmission > 0
// (BasicMaterial::adjustDoubleSidedFlag, BasicMaterial.cpp:719-731)
bool recordDoubleSided(const plt_material_record& r) {
    return (r.flags & PLT_MATERIAL_FLAG_DOUBLE_SIDED) != 0 || half_to_float(r.specular_transmission) > 0.f ||
           half_to_float(r.diffuse_transmission) > 0.f;
}
bool isDoubleSided(const Scene& s, uint32_t m) { return s.matFlags[m] != 0; }

// prepareShadingData, MaterialFactory.slang:79-128 with computeTangentSpace / orthonormalizeSafe
// (ShadingUtils.slang:126-153,243-251); opacity = evalOpacity of the PLT materials (.5 * alpha,
// PLTDiffuse: alpha).  No normal maps.
ShadingData prepareShadingData(const Scene& s, const VertexData& v, uint32_t materialID, F3 viewDir) {
    ShadingData sd;
    sd.posW = v.posW;
    sd.V = viewDir;
    sd.N = v.normalW;
    const F3 t = {v.tangentW[0], v.tangentW[1], v.tangentW[2]};
    const float NdotT = dot(t, sd.N);
    const bool nonParallel = std::fabs(NdotT) < 0.9999f;
    const bool nonZero = dot(t, t) > 0.f;
    const bool valid = std::fabs(v.tangentW[3]) == 1.0f && nonZero && nonParallel;
    if (valid) {
        sd.T = normalize(t - sd.N * NdotT);
        sd.B = cross(sd.N, sd.T) * v.tangentW[3];
    } else {
        sd.T = perp_stark(sd.N);
        sd.B = cross(sd.N, sd.T);
    }
    sd.faceN = v.faceNormalW;
    sd.frontFacing = dot(sd.V, sd.faceN) >= 0.f;
    sd.materialID = materialID;
    const Material<float>& m = s.mats[materialID];
    sd.opacity = m.type == PLT_MATERIAL_DIFFUSE ? m.base[3] : .5f * m.base[3];
    if (!sd.frontFacing && isDoubleSided(s, materialID)) sd.N = -sd.N;
    return sd;
}

// ---------------------------------------------------------------------------------------------
// Material instance in world space: the IMaterialInstance wrappers (PLT*BSDF.slang), with the
// grated materials working in the grating shading frame (DiffractionGrating.slang:83-90).
// ---------------------------------------------------------------------------------------------
template <class Fn> void withBx(const Material<float>& m, const SceneTables& tb, Fn&& fn) {
    const V2<float> none = {1.f, 0.f};
    switch (m.type) {
    case PLT_MATERIAL_DIFFUSE: { Diffuse<float> b(m); fn(b, false, none); return; }
    case PLT_MATERIAL_CONDUCTOR: { Conductor<float> b(m, &tb); fn(b, false, none); return; }
    case PLT_MATERIAL_DIELECTRIC: { Dielectric<float> b(m); fn(b, false, none); return; }
    case PLT_MATERIAL_OPAQUE_DIELECTRIC: { OpaqueDielectric<float> b(m); fn(b, false, none); return; }
    case PLT_MATERIAL_THIN_DIELECTRIC: { ThinDielectric<float> b(m); fn(b, false, none); return; }
    case PLT_MATERIAL_COATED_CONDUCTOR: { Coated<float, true> b(m, &tb); fn(b, false, none); return; }
    case PLT_MATERIAL_COATED_OPAQUE_DIELECTRIC: { Coated<float, false> b(m, &tb); fn(b, false, none); return; }
    case PLT_MATERIAL_GRATED_CONDUCTOR: { Grated<float, true> b(m, &tb); fn(b, true, b.grating.gratingX); return; }
    case PLT_MATERIAL_GRATED_OPAQUE_DIELECTRIC: { Grated<float, false> b(m, &tb); fn(b, true, b.grating.gratingX); return; }
    case PLT_MATERIAL_MULTILAYERED_STACK: { MultiLayer<float> b(m); fn(b, false, none); return; }
    default: return;
    }
}

Frame<float> sdFrame(const ShadingData& sd) { return {sd.T, sd.B, sd.N}; }
// localGratingShadingFrame, DiffractionGrating.slang:83-90
Frame<float> gratingSdFrame(const ShadingData& sd, V2<float> gx) {
    Frame<float> f;
    f.T = sd.fromLocal(F3{gx.x, gx.y, 0.f});
    f.N = sd.N;
    f.B = cross(f.N, f.T);
    return f;
}

struct BSDFSample {
    F3 wo = {0.f, 0.f, 0.f};
    float pdf = 0.f, weight = 0.f;
    uint32_t lobe = 0;
};

void bsdfEval(const Scene& s, const ShadingData& sd, F3 toEye, uint32_t lobe, Beam<float>& beam) {
    withBx(s.mats[sd.materialID], s.tables, [&](auto& bx, bool grated, V2<float> gx) {
        const Frame<float> F = grated ? gratingSdFrame(sd, gx) : sdFrame(sd);
        beam.r = F.toLocal(beam.r);
        beam.t = F.toLocal(beam.t);
        const F3 wiL = F.toLocal(sd.V), woL = F.toLocal(toEye);
        beam.constructLocalFrame(woL);
        bx.eval(wiL, woL, lobe, beam);
        beam.transformCoherence(bx.coherenceTransform(wiL, woL, lobe));
        beam.r = F.fromLocal(beam.r);
        beam.t = F.fromLocal(beam.t);
    });
}
bool bsdfSampleHint(const Scene& s, const ShadingData& sd, SampleGen& sg, BSDFSample& out, float wavelength, uint32_t lobeMask, F3 woHint);
// sample(sd, sg, result, wavelength): lobe mask All, no hint (the sample pass)
bool bsdfSample(const Scene& s, const ShadingData& sd, SampleGen& sg, BSDFSample& out, float wavelength) {
    return bsdfSampleHint(s, sd, sg, out, wavelength, LOBE_ALL, F3{0.f, 0.f, 0.f});
}
// sample(sd, sg, result, wavelength, lobeMask, woHint) of the wrappers: the dielectric and the thin
// dielectric restrict the lobes to the hint's side (PLTDielectricBSDF.slang:310-321,
// PLTThinDielectricBSDF.slang:230-243), the grated materials pick the diffraction order closest to
// the hint, the others ignore it.
bool bsdfSampleHint(const Scene& s, const ShadingData& sd, SampleGen& sg, BSDFSample& out, float wavelength, uint32_t lobeMask, F3 woHint) {
    bool valid = false;
    const Material<float>& m = s.mats[sd.materialID];
    withBx(m, s.tables, [&](auto& bx, bool grated, V2<float> gx) {
        const Frame<float> F = grated ? gratingSdFrame(sd, gx) : sdFrame(sd);
        if (m.type == PLT_MATERIAL_DIELECTRIC || m.type == PLT_MATERIAL_THIN_DIELECTRIC) {
            const float dh = dot(sd.V, woHint);
            const uint32_t lobes = (dh > 0.f ? LOBE_REFLECTION : dh < 0.f ? LOBE_TRANSMISSION : LOBE_ALL) & lobeMask;
            valid = bx.sample(F.toLocal(sd.V), out.wo, out.pdf, out.weight, out.lobe, sg, wavelength, lobes);
            if (valid || m.type == PLT_MATERIAL_DIELECTRIC) out.wo = F.fromLocal(out.wo);
            return;
        }
        if constexpr (std::is_same_v<std::decay_t<decltype(bx)>, Grated<float, true>> ||
                      std::is_same_v<std::decay_t<decltype(bx)>, Grated<float, false>>) {
            valid = bx.sampleHint(F.toLocal(sd.V), out.wo, out.pdf, out.weight, out.lobe, sg, wavelength, lobeMask, F.toLocal(woHint));
        } else {
            valid = bx.sample(F.toLocal(sd.V), out.wo, out.pdf, out.weight, out.lobe, sg, wavelength, lobeMask);
        }
        if (valid) out.wo = F.fromLocal(out.wo);
    });
    return valid;
}

// ---------------------------------------------------------------------------------------------
// Differential shading geometry and scattering derivatives for manifold walks,
// Rendering/Utils/DifferentialShadingGeometry.slang:28-222
// ---------------------------------------------------------------------------------------------
struct F3pdv { F3 v, ddu, ddv; };
struct F3kpdv { F3 v, ddu, ddv, ddl; };
struct DSG {
    F3pdv p, n, s, t;
    F3 fromLocal(F3 v) const { return s.v * v.x + t.v * v.y + n.v * v.z; }
    // pdw: direction from the surface point to dst and its derivatives
    F3pdv pdw(F3 dst) const {
        F3pdv w;
        w.v = dst - p.v;
        const float ilo = 1.f / length(w.v);
        w.v = w.v * ilo;
        w.ddu = (p.ddu - w.v * dot(w.v, p.ddu)) * -ilo;
        w.ddv = (p.ddv - w.v * dot(w.v, p.ddv)) * -ilo;
        return w;
    }
};
F3 zero3() { return {0.f, 0.f, 0.f}; }
// differentialShadingGeometry (untextured: the (1,0), (0,1) triangle parameterisation)
DSG differentialShadingGeometry(const Scene& s, uint32_t prim, float b1, float b2) {
    const float bary[3] = {1.f - b1 - b2, b1, b2};
    const uint32_t* I = s.idx + 3 * (size_t)prim;
    const F3 p0 = f3(s.pos + 3 * (size_t)I[0]), p1 = f3(s.pos + 3 * (size_t)I[1]), p2 = f3(s.pos + 3 * (size_t)I[2]);
    const F3 n0 = f3(s.nrm + 3 * (size_t)I[0]), n1 = f3(s.nrm + 3 * (size_t)I[1]), n2 = f3(s.nrm + 3 * (size_t)I[2]);
    DSG g;
    g.p.v = p0 * bary[0] + p1 * bary[1] + p2 * bary[2];
    g.n.v = n0 * bary[0] + n1 * bary[1] + n2 * bary[2];
    const float il = 1.0f / length(g.n.v);
    g.n.v = g.n.v * il;
    g.p.ddu = perp_stark(g.n.v);
    g.p.ddv = cross(g.n.v, g.p.ddu);
    const float duv0x = 1.f, duv0y = 0.f, duv1x = 0.f, duv1y = 1.f;
    const F3 dp0 = p1 - p0, dp1 = p2 - p0;
    g.n.ddu = (n1 - n0) * il;
    g.n.ddv = (n2 - n0) * il;
    g.n.ddu = g.n.ddu - g.n.v * dot(g.n.v, g.n.ddu);
    g.n.ddv = g.n.ddv - g.n.v * dot(g.n.v, g.n.ddv);
    const float det = duv0x * duv1y - duv0y * duv1x;
    if (std::fabs(det) > K_FLT_EPSILON) {
        const float invDet = 1.0f / det;
        g.p.ddu = (dp0 * duv1y - dp1 * duv0y) * invDet;
        g.p.ddv = (dp0 * -duv1x + dp1 * duv0x) * invDet;
        const F3 nddu = (g.n.ddu * duv1y - g.n.ddv * duv0y) * invDet;
        const F3 nddv = (g.n.ddu * -duv1x + g.n.ddv * duv0x) * invDet;
        g.n.ddu = nddu;
        g.n.ddv = nddv;
    } else {
        g.n.ddu = zero3();
        g.n.ddv = zero3();
    }
    g.s.v = g.p.ddu - g.n.v * dot(g.n.v, g.p.ddu);
    float ils = 1.0f / length(g.s.v);
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
F3kpdv reflectDerivatives(const F3pdv& wi, const F3pdv& n) {
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
F3kpdv refractDerivatives(const F3pdv& wi, F3pdv n, float eta) {
    const float wn = dot(wi.v, n.v);
    eta = wn < 0.f ? eta : 1.f / eta;
    const float dEdl = 0.f;
    if (wn < 0.f) { n.v = -n.v; n.ddu = -n.ddu; n.ddv = -n.ddv; }
    const float eta2 = sqr(eta);
    const float dwdun = dot(wi.ddu, n.v), dwdvn = dot(wi.ddv, n.v);
    const float dnduw = dot(n.ddu, wi.v), dndvw = dot(n.ddv, wi.v);
    const float root = std::sqrt(std::max(0.f, 1.f - eta2 * (1.0f - sqr(wn))));
    F3kpdv r;
    if (root == 0.f) { r.v = r.ddu = r.ddv = r.ddl = zero3(); return r; }
    const float dRoot = -(1.0f - sqr(wn)) * eta * dEdl / root;
    const float a = eta - eta2 * wn / root;
    r.v = (wi.v - n.v * wn) * -eta - n.v * root;
    r.ddu = n.v * (a * (dnduw + dwdun)) + n.ddu * (eta * wn - root) - wi.ddu * eta;
    r.ddv = n.v * (a * (dndvw + dwdvn)) + n.ddv * (eta * wn - root) - wi.ddv * eta;
    r.ddl = (wi.v - n.v * wn) * -dEdl - n.v * dRoot;
    return r;
}
// DiffractionGrating.partialDerivatives, DiffractionGrating.slang:188-265
F3kpdv gratingDerivatives(const DSG& g, const F3pdv& wi, V2<float> gx, V2<float> invPitch, int lx, int ly, float wavelength) {
    F3kpdv ret;
    ret.v = ret.ddu = ret.ddv = ret.ddl = zero3();
    const F3pdv& n = g.n;
    F3pdv X;
    X.v = g.fromLocal(F3{gx.x, gx.y, 0.f});
    X.ddu = g.s.ddu * gx.x + g.t.ddu * gx.y;
    X.ddv = g.s.ddv * gx.x + g.t.ddv * gx.y;
    if (lx == 0 && ly == 0) return reflectDerivatives(wi, n);
    const float lambda = 1e-3f * wavelength;
    const float lpx = (float)lx * invPitch.x, lpy = (float)ly * invPitch.y;
    const F3 Y = cross(n.v, X.v);
    const float x = dot(wi.v, X.v), y = dot(wi.v, Y), z = dot(wi.v, n.v);
    const float px = std::sqrt(sqr(x) + sqr(z)), py = std::sqrt(sqr(y) + sqr(z));
    const float ipx = px > K_FLT_EPSILON ? 1.f / px : 0.f, ipy = py > K_FLT_EPSILON ? 1.f / py : 0.f;
    const float sinix = x * ipx, siniy = y * ipy;
    const float a = lambda * lpx - sinix, b = lambda * lpy - siniy;
    const float oneMinusA2 = std::max(0.f, 1 - sqr(a));
    const float m = -oneMinusA2 / (sqr(a * b) - 1);
    const float q = 1 - sqr(b) * m;
    if (a > 1.f || a < -1.f || b > 1.f || b < -1.f || q < 0.f || !(m >= 0.f)) return ret;
    const float sqrtOneM = std::sqrt(q), sqrtM = std::sqrt(m);
    const float c = .5f / (sqrtOneM * std::sqrt(oneMinusA2));
    const float dxdu = dot(wi.v, X.ddu) + dot(wi.ddu, X.v), dxdv = dot(wi.v, X.ddv) + dot(wi.ddv, X.v);
    const float dzdu = dot(wi.v, n.ddu) + dot(wi.ddu, n.v), dzdv = dot(wi.v, n.ddv) + dot(wi.ddv, n.v);
    const float dadu = z * (x * dzdu - z * dxdu) * (sqr(ipx) * ipx);
    const float dbdu = z * (y * dzdu - z * dxdu) * (sqr(ipy) * ipy);
    const float dadv = z * (x * dzdv - z * dxdv) * (sqr(ipx) * ipx);
    const float dbdv = z * (y * dzdv - z * dxdv) * (sqr(ipy) * ipy);
    const float dadl = lpx, dbdl = lpy;
    const float den = sqr(sqr(a * b) - 1);
    const float dmdu = 2 * a * (a * b * oneMinusA2 * dbdu - dadu * (1 - sqr(b))) / den;
    const float dmdv = 2 * a * (a * b * oneMinusA2 * dbdv - dadv * (1 - sqr(b))) / den;
    const float dmdl = 2 * a * (a * b * oneMinusA2 * dbdl - dadl * (1 - sqr(b))) / den;
    ret.v = X.v * (a * sqrtOneM) + Y * (b * sqrtM) + n.v * std::sqrt(std::max(0.f, 1 - sqr(a) * q - sqr(b) * m));
    auto d = [&](float da, float db, float dm) {
        return X.v * ((q * da - a * b * (b * dm / 2.f + m * db)) / sqrtOneM) + Y * ((b * dm / 2.f + m * db) / sqrtM) +
               n.v * ((-2 * a * da * q - b * (b * dm + 2.f * m * db) + sqr(a) * b * (b * dm + 2.f * m * db)) * c);
    };
    ret.ddu = d(dadu, dbdu, dmdu);
    ret.ddv = d(dadv, dbdv, dmdv);
    ret.ddl = d(dadl, dbdl, dmdl);
    return ret;
}
// IMaterialInstance.partialDerivatives of each PLT*BSDF.slang (world space)
F3kpdv bsdfPartialDerivatives(const Scene& s, uint32_t mid, const F3pdv& wi, const DSG& g, uint32_t lobe, float wavelength) {
    const Material<float>& m = s.mats[mid];
    switch (m.type) {
    case PLT_MATERIAL_DIELECTRIC: {
        Dielectric<float> b(m);
        if (lobe & LOBE_TRANSMISSION) {
            const float k = (float)K_2PI / (1e-3f * wavelength);
            return refractDerivatives(wi, g.n, b.ior(k));
        }
        return reflectDerivatives(wi, g.n);
    }
    case PLT_MATERIAL_THIN_DIELECTRIC:
        if (lobe & LOBE_TRANSMISSION) {
            F3kpdv r;
            r.v = -wi.v; r.ddu = -wi.ddu; r.ddv = -wi.ddv; r.ddl = zero3();
            return r;
        }
        return reflectDerivatives(wi, g.n);
    case PLT_MATERIAL_GRATED_CONDUCTOR:
    case PLT_MATERIAL_GRATED_OPAQUE_DIELECTRIC: {
        int lx, ly;
        decodeGratingLobe(lobe, lx, ly);
        if (lx == 0 && ly == 0) return reflectDerivatives(wi, g.n);
        const DiffractionGrating<float> gr = makeGrating(m);
        return gratingDerivatives(g, wi, gr.gratingX, gr.invPitch, lx, ly, wavelength);
    }
    case PLT_MATERIAL_DIFFUSE: {
        F3kpdv r;
        r.v = r.ddu = r.ddv = r.ddl = zero3();
        return r;
    }
    default: return reflectDerivatives(wi, g.n);
    }
}

// sphcoords / derivatives and one Newton step on the angle constraint, Manifolds.slangh:283-347
void sphcoords(F3 w, float& theta, float& phi) {
    theta = std::acos(std::min(std::max(w.z, -1.f), 1.f));
    phi = std::atan2(w.y, w.x);
    phi += phi < 0.f ? (float)K_2PI : 0.f;
}
bool manifoldOneStep(const F3pdv& w, const F3kpdv& ws, const F3pdv& p, float& lenC, F3& stepDir) {
    float t0, p0, t1, p1;
    sphcoords(w.v, t0, p0);
    sphcoords(ws.v, t1, p1);
    const float dt = t0 - t1;
    float dp = p0 - p1;
    dp = std::fabs(dp) > (float)K_PI ? dp - o_sign(dp) * (float)K_2PI : dp;
    lenC = std::sqrt(dt * dt + dp * dp);
    auto der = [](F3 v, F3 du, F3 dv, float out[2][2]) {
        const float dAcos = -1.f / std::sqrt(std::max(0.f, 1.f - sqr(v.z)));
        const float invNorm = 1.f / (v.x * v.x + v.y * v.y);
        out[0][0] = dAcos * du.z;
        out[0][1] = dAcos * dv.z;
        out[1][0] = invNorm * (v.x * du.y - v.y * du.x);
        out[1][1] = invNorm * (v.x * dv.y - v.y * dv.x);
    };
    float dO[2][2], dI[2][2];
    der(w.v, w.ddu, w.ddv, dO);
    der(ws.v, ws.ddu, ws.ddv, dI);
    const float A = dO[0][0] - dI[0][0], B = dO[0][1] - dI[0][1], C = dO[1][0] - dI[1][0], D = dO[1][1] - dI[1][1];
    // tryInvert with the reference's determinant threshold, MathHelpers.slang:484-498
    const float det = A * D - B * C;
    if (std::fabs(det) < 4e-6f) return false;
    const float id = 1.f / det;
    const float i00 = D * id, i01 = -B * id, i10 = -C * id, i11 = A * id;
    const float dx = i00 * dt + i01 * dp, dy = i10 * dt + i11 * dp;
    stepDir = p.ddu * dx + p.ddv * dy;
    return true;
}

struct MSHit {
    uint32_t prim;
    float b1, b2;
    F3 posW;
    uint32_t lobe;
};
struct ManifoldSample {
    MSHit hits[4];
    F3 woLastHitToLight = {0.f, 0.f, 0.f};
    int hitCount = 0;
    uint32_t iterations = 0;
    float wavelength = 0.f;
    float pdf = 1.f;
    bool dispersive = false;
};

float bsdfPdf(const Scene& s, const ShadingData& sd, F3 toLight, float wavelength) {
    float p = 0.f;
    withBx(s.mats[sd.materialID], s.tables, [&](auto& bx, bool grated, V2<float> gx) {
        const Frame<float> F = grated ? gratingSdFrame(sd, gx) : sdFrame(sd);
        p = bx.pdf(F.toLocal(toLight), F.toLocal(sd.V), wavelength);
    });
    return p;
}
void bsdfLambdaPdf(const Scene& s, const ShadingData& sd, F3 wo, uint32_t lobe, const Beam<float>& beamIn, float* out) {
    withBx(s.mats[sd.materialID], s.tables, [&](auto& bx, bool, V2<float>) {
        Beam<float> b = beamIn;
        b.r = sd.toLocal(b.r);
        b.t = sd.toLocal(b.t);
        bx.lambdaPdf(sd.toLocal(sd.V), sd.toLocal(wo), lobe, b, out);
    });
}

// Learned proposal features of a material (roughness, pitch feature, class, enabled), as the
// library's material upload derives them: classes conductor 0, dielectric 1, opaque dielectric 2,
// coated conductor 3, coated opaque dielectric 4, grated conductor 5, grated opaque dielectric 6,
// diffuse 7; enabled for materials with non-delta lobes other than PLTDiffuse.  The roughness
// feature is the surface model's q, the pitch feature the grating pitch x in um / 5.
void proposalFeatures(const Material<float>& m, const SceneTables& t, float* f) {
    float rough = 0.f, pitch = 0.f, cls = -1.f;
    bool scatter = false;
    switch (m.type) {
    case PLT_MATERIAL_CONDUCTOR: cls = 0.f; rough = Conductor<float>(m, &t).gfs.q(); scatter = true; break;
    case PLT_MATERIAL_DIELECTRIC: cls = 1.f; rough = Dielectric<float>(m).gfs.q; scatter = rough != 0.f; break;
    case PLT_MATERIAL_OPAQUE_DIELECTRIC: cls = 2.f; rough = OpaqueDielectric<float>(m).gfs.q(); scatter = true; break;
    case PLT_MATERIAL_COATED_CONDUCTOR: cls = 3.f; rough = Coated<float, true>(m, &t).gfs.q(); scatter = true; break;
    case PLT_MATERIAL_COATED_OPAQUE_DIELECTRIC: cls = 4.f; rough = Coated<float, false>(m, &t).gfs.q(); scatter = true; break;
    case PLT_MATERIAL_GRATED_CONDUCTOR:
    case PLT_MATERIAL_GRATED_OPAQUE_DIELECTRIC: {
        cls = m.type == PLT_MATERIAL_GRATED_CONDUCTOR ? 5.f : 6.f;
        rough = OpaqueDielectric<float>(m, true).gfs.q();
        const DiffractionGrating<float> g = makeGrating(m);
        pitch = g.invPitch.x > 0.f ? (1.f / g.invPitch.x) / 5.f : 0.f;
        scatter = true;
        break;
    }
    case PLT_MATERIAL_DIFFUSE: cls = 7.f; rough = 1.f; break;
    default: break;
    }
    f[0] = rough;
    f[1] = pitch;
    f[2] = cls;
    f[3] = scatter ? 1.f : 0.f;
}

// getProperties / getLobes of each PLT*BSDF.slang
struct Props {
    uint32_t flags = 0;
    uint32_t emissionId = PLT_NO_SPECTRAL_PROFILE;
    uint32_t lobes = 0;
};
Props bsdfProps(const Scene& s, uint32_t materialID) {
    const Material<float>& m = s.mats[materialID];
    Props p;
    auto rough = [](float q, uint32_t deltaLobes, uint32_t scatterLobes) { return q == 0.f ? deltaLobes : (deltaLobes | scatterLobes); };
    switch (m.type) {
    case PLT_MATERIAL_DIFFUSE:
        p.emissionId = m.emission;
        p.flags = m.emission != PLT_NO_SPECTRAL_PROFILE ? PROP_EMISSIVE : 0u;
        p.lobes = LOBE_DIFFUSE_REFLECTION;
        break;
    case PLT_MATERIAL_DIELECTRIC: {
        Dielectric<float> b(m);
        p.flags = PROP_TRANSMISSIVE | (b.gfs.q < kQcutoffForMS ? PROP_MW_TRANSMISSIVE : 0u);
        const uint32_t dt = b.isDispersive() ? LOBE_DISPERSIVE_DELTA_TRANSMISSION : LOBE_DELTA_TRANSMISSION;
        p.lobes = rough(b.gfs.q, LOBE_DELTA_REFLECTION | dt, LOBE_SCATTER_REFLECTION | LOBE_SCATTER_TRANSMISSION);
        break;
    }
    case PLT_MATERIAL_CONDUCTOR: {
        Conductor<float> b(m, &s.tables);
        p.flags = b.gfs.q() < kQcutoffForMS ? PROP_MW_REFLECTIVE : 0u;
        p.lobes = rough(b.gfs.q(), LOBE_DELTA_REFLECTION, LOBE_SCATTER_REFLECTION);
        break;
    }
    case PLT_MATERIAL_OPAQUE_DIELECTRIC: {
        OpaqueDielectric<float> b(m);
        p.flags = b.gfs.q() < kQcutoffForMS ? PROP_MW_REFLECTIVE : 0u;
        p.lobes = rough(b.gfs.q(), LOBE_DELTA_REFLECTION, LOBE_SCATTER_REFLECTION);
        break;
    }
    case PLT_MATERIAL_COATED_CONDUCTOR:
    case PLT_MATERIAL_COATED_OPAQUE_DIELECTRIC: {
        Coated<float, true> b(m, &s.tables);
        p.flags = b.gfs.q() < kQcutoffForMS ? PROP_MW_REFLECTIVE : 0u;
        p.lobes = rough(b.gfs.q(), LOBE_DELTA_REFLECTION, LOBE_SCATTER_REFLECTION);
        break;
    }
    case PLT_MATERIAL_GRATED_CONDUCTOR: {
        Grated<float, true> b(m, &s.tables);
        p.flags = PROP_MW_REFLECTIVE;
        p.lobes = rough(b.baseC.gfs.q(), LOBE_DELTA_REFLECTION, LOBE_SCATTER_REFLECTION) | LOBE_DISPERSIVE_DELTA_REFLECTION;
        break;
    }
    case PLT_MATERIAL_GRATED_OPAQUE_DIELECTRIC: {
        Grated<float, false> b(m, &s.tables);
        p.flags = PROP_MW_REFLECTIVE;
        p.lobes = rough(b.baseD.gfs.q(), LOBE_DELTA_REFLECTION, LOBE_SCATTER_REFLECTION) | LOBE_DISPERSIVE_DELTA_REFLECTION;
        break;
    }
    case PLT_MATERIAL_THIN_DIELECTRIC:
        p.flags = PROP_TRANSMISSIVE | PROP_MW_REFLECTIVE | PROP_MW_TRANSMISSIVE;
        p.lobes = LOBE_DELTA_REFLECTION | LOBE_DELTA_TRANSMISSION;
        break;
    case PLT_MATERIAL_MULTILAYERED_STACK:
        p.flags = PROP_MW_REFLECTIVE;
        p.lobes = LOBE_DELTA_REFLECTION;
        break;
    default: break;
    }
    return p;
}

// ---------------------------------------------------------------------------------------------
// Spectra: SpectrumSampler (SpectrumSampler.slang:38-54), Scene.sampleSpectrum (Scene.slang:295-330),
// spectrumToRgb (SpectrumUtils.slang:43-104, ColorHelpers.slang:61-70)
// ---------------------------------------------------------------------------------------------
constexpr float kMinWl = 380.0f, kMaxWl = 720.0f;
float sampleOneWavelength(float u) { return kMinWl + u * (kMaxWl - kMinWl); }
void hwssWavelengths(float hero, uint32_t H, float* out) {
    const float span = kMaxWl - kMinWl;
    for (uint32_t i = 0; i < H; ++i) {
        float w = hero + float(i) * (span / float(H));
        w -= w > kMaxWl ? span : 0.f;
        out[i] = w;
    }
}
// returns Le per hwss sample; sampled wavelengths in wl
void sampleSpectrum(const Scene& s, uint32_t id, float hero, SampleGen& sg, bool importance, uint32_t H, float* le, float* wl) {
    for (uint32_t j = 0; j < H; ++j) le[j] = 0.f;
    if (id == PLT_NO_SPECTRAL_PROFILE || id >= s.tables.count) return;   // sampledWavelengths stays unset in the reference
    if (importance) {
        const plt_spectral_profile& sp = s.tables.profiles[id];
        wl[0] = hero;
        le[0] = evalSpectrum<float>(s.tables, id, hero);
        // three draws (sampleNext3D) for at most three companions; beyond HWSS 4 one per companion
        const uint32_t draws = H - 1 > 3 ? H - 1 : 3;
        float x[MAXH];
        for (uint32_t c = 0; c < draws; ++c) x[c] = float(sp.bins) * sg.next1D();
        for (uint32_t j = 1; j < H; ++j) {
            const uint32_t i = (uint32_t)x[j - 1];
            const float a = i < sp.bins ? sp.icdf[i] : 1.f;
            const float b = i + 1 < sp.bins ? sp.icdf[i + 1] : 1.f;
            const float fr = x[j - 1] - std::floor(x[j - 1]);
            const float cdf = a + (b - a) * fr;
            wl[j] = sp.min_wavelength + (sp.max_wavelength - sp.min_wavelength) * cdf;
            le[j] = sp.intensity / (float)sp.bins;
        }
    } else {
        hwssWavelengths(hero, H, wl);
        for (uint32_t j = 0; j < H; ++j) le[j] = evalSpectrum<float>(s.tables, id, wl[j]);
    }
}
F3 spectrumToRgb(const float* L, const float* wl, uint32_t samples) {
    F3 res = {0.f, 0.f, 0.f};
    for (uint32_t i = 0; i < samples; ++i) {
        const F3 xyz = wavelengthToXYZ(wl[i]) * wavelengthToD65(wl[i]) * L[i];
        const F3 rgb = {3.240969941904522f * xyz.x + -1.537383177570094f * xyz.y + -0.4986107602930032f * xyz.z,
                        -0.9692436362808803f * xyz.x + 1.875967501507721f * xyz.y + 0.04155505740717569f * xyz.z,
                        0.05563007969699373f * xyz.x + -0.2039769588889765f * xyz.y + 1.056971514242878f * xyz.z};
        res = res + rgb;
    }
    const float Y_D65 = 10.5670762f;
    return res / Y_D65;
}

// ---------------------------------------------------------------------------------------------
// Beams: pltSourceBeamArea (PLT.slang:276-290) and propagate (PLT.slang:224-230)
// ---------------------------------------------------------------------------------------------
Beam<float> sourceBeamArea(F3 posW, F3 dir, float A, float dist, const float* Le, const float* wl, uint32_t H, float maxBeamOmega) {
    const float r2 = sqr(dist * 1e+3f);
    A = std::min(A, maxBeamOmega * r2);
    Beam<float> b;
    b.H = (int)H;
    for (uint32_t j = 0; j < H; ++j) {
        b.L[0][j] = Le[j];
        b.L[1][j] = b.L[2][j] = b.L[3][j] = 0.f;
        b.wl[j] = wl[j];
        b.spdf[j] = 1.f;
    }
    b.D[0] = A; b.D[1] = 0.f; b.D[2] = A;
    b.r_m = 0.f;
    b.posW = posW;
    b.r = dir;
    b.t = perp_stark(dir);
    b.distant = false;
    return b;
}
// pltSourceBeamDistant (PLT.slang:253-267): diffusivity min(solidAngle, maxOmega) I, coherence
// radius 1 mm, distant for the beam's whole life
Beam<float> sourceBeamDistant(F3 dir, float solidAngle, const float* Le, const float* wl, uint32_t H, float maxBeamOmega) {
    solidAngle = std::min(solidAngle, maxBeamOmega);
    Beam<float> b;
    b.H = (int)H;
    for (uint32_t j = 0; j < H; ++j) {
        b.L[0][j] = Le[j];
        b.L[1][j] = b.L[2][j] = b.L[3][j] = 0.f;
        b.wl[j] = wl[j];
        b.spdf[j] = 1.f;
    }
    b.D[0] = solidAngle; b.D[1] = 0.f; b.D[2] = solidAngle;
    b.r_m = 1e-3f;
    b.posW = {0.f, 0.f, 0.f};
    b.r = dir;
    b.t = perp_stark(dir);
    b.distant = true;
    return b;
}
void propagate(Beam<float>& b, F3 p) {
    if (!b.distant) b.r_m += length(p - b.posW);
    b.posW = p;
}
void scaleBeam(Beam<float>& b, float s) {
    for (int c = 0; c < 4; ++c) for (int j = 0; j < b.H; ++j) b.L[c][j] *= s;
}

float MISWeight(float p0, float p1) {
    const float q0 = p0, q1 = p1;
    return q0 / (q0 + q1);
}

// ---------------------------------------------------------------------------------------------
// The render pass
// ---------------------------------------------------------------------------------------------
struct Renderer {
    const Scene& s;
    const plt_camera& cam;
    Options o;
    uint32_t width, height, frame;

    uint32_t trace(F3 org, F3 dir, float t0, float t1, float& t, float& b1, float& b2) const {
        const float O[3] = {org.x, org.y, org.z}, D[3] = {dir.x, dir.y, dir.z};
        return s.bvh.trace(O, D, t0, t1, false, t, b1, b2);
    }
    bool visible(F3 org, F3 dir, float t0, float t1) const {
        const float O[3] = {org.x, org.y, org.z}, D[3] = {dir.x, dir.y, dir.z};
        float t, b1, b2;
        return s.bvh.trace(O, D, t0, t1, true, t, b1, b2) == kNone;
    }

    // Camera.computeRayPinhole, Camera.slang:46-78
    F3 cameraDir(uint32_t px, uint32_t py) const {
        float p0 = (float(px) + 0.5f) / float(width);
        float p1 = (float(py) + 0.5f) / float(height);
        p0 += -cam.jitter_x;
        p1 += cam.jitter_y;
        const float ndcx = 2.f * p0 + -1.f, ndcy = -2.f * p1 + 1.f;
        const F3 d = f3(cam.u) * ndcx + f3(cam.v) * ndcy + f3(cam.w);
        return normalize(d);
    }

    // ---- sample pass, pltpt_sample.rt.slang:36-185 ----
    void samplePass(uint32_t px, uint32_t py, Bounce* bounces) const {
        SampleGen sg(px, py, frame, o.tinySg);
        const float wavelength = sampleOneWavelength(sg.next1D());
        F3 origin = f3(cam.pos), dir = cameraDir(px, py);
        float weight = 1.f, pdf = 1.f, thp = 1.f, lastNonDeltaPdf = 0.f;
        float wps = 1.f;   // product of the primary-sample MIS densities (learned proposal)
        uint32_t flags = FLAG_ONLY_DELTA;
        const uint32_t maxB = o.maxBounces;
        auto append = [&](uint32_t length, uint32_t prim, float b1, float b2, F3 wi, uint32_t lobe, uint32_t extra = 0u) {
            Bounce& b = bounces[length];
            b.flags = flags | extra;
            b.prim = prim;
            b.b1 = b1;
            b.b2 = b2;
            const float n[3] = {wi.x, wi.y, wi.z};
            geom::ndirToOctEqualArea(n, b.ewi);
            b.lobe = lobe;
            b.lastNonDeltaPdf = lastNonDeltaPdf;
            b.pathContribution = 1.f / (pdf * thp * wps);
        };
        for (uint32_t length = 0; length < maxB + 1 && (flags & (FLAG_MISS | FLAG_TERMINATED)) == 0;) {
            float t, b1, b2;
            const uint32_t prim = trace(origin, dir, 0.f, FLT_MAX, t, b1, b2);
            const F3 wi = -dir;
            if (prim == kNone) {       // scatterMiss
                flags |= FLAG_MISS;
                append(length, kNone, 0.f, 0.f, wi, 0);
                continue;
            }
            // scatterTriangleMeshClosestHit
            const VertexData v = vertexData(s, prim, b1, b2);
            const uint32_t mid = s.triMat[prim];
            const ShadingData sd = prepareShadingData(s, v, mid, wi);
            const Props props = bsdfProps(s, mid);
            if (o.alphaMask && sd.opacity == 0.f) {   // alpha mask (kAlphaMasking)
                origin = sd.newRayOrigin(false);
                continue;
            }
            // shouldTerminatePath: RR(1 - weight, 2, u), pltpt.slangh:170-176; pow follows the
            // shader semantics (NaN for a negative base)
            float rcp_thp = 1.f;
            if (o.doRR) {
                const float rrVal = 1.f - weight;
                const float p = rrVal < 0.f ? NAN : std::pow(rrVal, 2.f);
                const float u = sg.next1D();
                rcp_thp = u < p ? 0.f : 1.f - p;
            }
            bool shouldEnd = length == maxB || (rcp_thp == 0.f && length > 0);
            // learned proposal (plt_pt.cuh ptBounceKernel<true>): a proposal vertex is an enabled
            // material hit from the front with wi above the shading plane; the network's mixture is
            // a density over the surface sampler's primary sample
            bool useNet = false;
            plt_oracle_mlp::PackedMix mix{};
            if (o.learned) {
                const float* mf = &s.matFeat[4 * (size_t)mid];
                const F3 wiL = sd.toLocal(sd.V);
                useNet = mf[3] > 0.f && sd.frontFacing && wiL.z > 0.f;
                if (useNet) {
                    double x[plt_oracle_mlp::kIn], z1[plt_oracle_mlp::kHid], z2[plt_oracle_mlp::kHid], z3[plt_oracle_mlp::kHid],
                        out[plt_oracle_mlp::kOut];
                    plt_oracle_mlp::featureRow(wiL.x, wiL.y, wiL.z, wavelength, mf, x);
                    s.net->forward(x, z1, z2, z3, out);
                    mix = plt_oracle_mlp::packMixture(out);
                }
            }
            const uint32_t extra = useNet ? FLAG_LEARNED : 0u;
            BSDFSample bs;
            float warp = 1.f;
            if (!shouldEnd) {
                // one-sample MIS in primary sample space: the surface sampler's primary sample comes
                // from the proposal (probability c) or is uniform; a non-delta direction's path weight
                // is divided by c q(u) + 1 - c, the analytic pdf is kept for everything else
                float warpU[2] = {0.f, 0.f};
                float mpss = 1.f;
                bool inside = true;
                if (useNet) {
                    const float c = o.learnedProb;
                    if (sg.next1D() < c) {
                        const float u0 = sg.next1D(), u1 = sg.next1D(), u2 = sg.next1D();
                        plt_oracle_mlp::sampleMixture(mix, u0, u1, u2, warpU[0], warpU[1]);
                        inside = warpU[0] >= 0.f && warpU[0] < 1.f && warpU[1] >= 0.f && warpU[1] < 1.f;
                    } else {
                        warpU[0] = sg.next1D();
                        warpU[1] = sg.next1D();
                    }
                    mpss = inside ? c * plt_oracle_mlp::mixtureDensity(mix, warpU[0], warpU[1]) + (1.f - c) : 0.f;
                    if (!inside) warpU[0] = warpU[1] = .5f;
                    g_directionWarp = warpU;
                }
                bool ok = bsdfSample(s, sd, sg, bs, wavelength);
                g_directionWarp = nullptr;
                if (useNet && ok && (bs.lobe & LOBE_DELTA) == 0) {
                    ok = inside && mpss > 0.f;
                    warp = mpss;
                }
                shouldEnd = !ok || bs.pdf == 0.f;
                const float nc = pdf * bs.pdf * thp * rcp_thp;
                shouldEnd = shouldEnd || nc < 1e-6f;
            }
            const bool isDelta = (bs.lobe & LOBE_DELTA) != 0;
            const bool isDisp = (bs.lobe & (LOBE_DISPERSIVE_DELTA_REFLECTION | LOBE_DISPERSIVE_DELTA_TRANSMISSION)) != 0;
            const bool isRefl = (bs.lobe & LOBE_REFLECTION) != 0;
            const bool isMS = (isRefl && (props.flags & PROP_MW_REFLECTIVE)) || (!isRefl && (props.flags & PROP_MW_TRANSMISSIVE));
            if (shouldEnd) {
                flags |= FLAG_TERMINATED;
                append(length, prim, b1, b2, wi, 0, extra);
                continue;
            }
            weight *= bs.weight;
            thp *= rcp_thp;
            pdf *= bs.pdf;
            wps *= warp;
            if (isDisp) flags |= FLAG_DISPERSIVE;
            append(length, prim, b1, b2, wi, bs.lobe, extra);
            ++length;
            lastNonDeltaPdf = !isDelta ? bs.pdf : lastNonDeltaPdf;
            const uint32_t msc = isMS ? (flags >> 16) + 1u : 0u;
            flags = (flags & 0xFFFFu) | (msc << 16);
            flags = isDelta ? (flags | FLAG_LAST_DELTA) : (flags & ~FLAG_LAST_DELTA);
            if (!isDelta) flags &= ~FLAG_ONLY_DELTA;
            origin = sd.newRayOrigin(isRefl);
            dir = bs.wo;
        }
    }

    // ---- solve pass, pltpt_solve.rt.slang ----
    struct Solve {
        SampleGen sg, tilesg;
        F3 Lrgb = {0.f, 0.f, 0.f};
        float dbg[4] = {0.f, 0.f, 0.f, 0.f};   // debugOutput (Path.slang:205)
        F3 pathOrigin, pathNormal;
        float wavelength = 0.f;
        uint64_t shadowRays = 0, unwindEvals = 0;
    };

    // wasNEEAvailable, pltpt_solve.rt.slang:204-210
    bool wasNEEAvailable(int p, uint32_t flags) const {
        return o.doNee && p > 0 &&
               ((flags & FLAG_LAST_DELTA) == 0 || (o.doMnee && (flags >> 16) <= o.mneeMaxOccluders && p > 1));
    }

    void forwardUnwindStep(uint32_t prim, const VertexData& v, F3 wo, uint32_t lobe, Beam<float>& beam, Solve& sv) const {
        const uint32_t mid = s.triMat[prim];
        const ShadingData sd = prepareShadingData(s, v, mid, -beam.r);
        propagate(beam, sd.posW);
        bsdfEval(s, sd, wo, lobe, beam);
        ++sv.unwindEvals;
        if (o.hwssMis) {
            float pdfs[MAXH];
            for (int j = 0; j < MAXH; ++j) pdfs[j] = 1.f;
            bsdfLambdaPdf(s, sd, wo, lobe, beam, pdfs);
            for (uint32_t j = 0; j < o.hwss; ++j) beam.spdf[j] *= pdfs[j];
        }
    }
    void forwardUnwind(int bounceIdx, const Bounce* bounces, Beam<float>& beam, Solve& sv) const {
        for (int p = bounceIdx - 1; p >= 0; --p) {
            const Bounce& b = bounces[p];
            const VertexData v = vertexData(s, b.prim, b.b1, b.b2);
            forwardUnwindStep(b.prim, v, b.wi(), b.lobe, beam, sv);
        }
    }

    // measure, pltpt_solve.rt.slang:96-147
    // writeDebugOutput, pltpt_debug.slangh:19-23
    void debugWrite(Solve& sv, uint32_t view, F3 v) const {
        if (o.debugView == view && std::isfinite(v.x) && std::isfinite(v.y) && std::isfinite(v.z)) {
            sv.dbg[0] += v.x;
            sv.dbg[1] += v.y;
            sv.dbg[2] += v.z;
            sv.dbg[3] += 1.f;
        }
    }

    void measure(Solve& sv, int bounceIdx, float pathContribution, Beam<float>& beam) const {
        if (!o.useDirect && bounceIdx <= 1) return;
        if (o.debugView) {
            // coherence views before the propagation to the camera (pltpt_solve.rt.slang:102-106);
            // coherenceAnisotropy through svd_symmetric (PLT.slang:193-197, MathHelpers.slang:583-605)
            const float k = float(K_2PI) / (1e-3f * beam.wl[0]);
            debugWrite(sv, PLT_DEBUG_VIEW_COHERENCE_AREA, colourCode(kMagma, std::sqrt(beam.coherenceArea(k)) / 150.f));
            const M2<float> A = beam.invTheta(k);
            const float a = A.m[0][0], b = A.m[1][0], c = A.m[0][1], d = A.m[1][1];
            const float a2 = a * a, b2 = b * b, c2 = c * c, d2 = d * d;
            const float y = 2.f * a * c + 2.f * b * d, x = a2 + b2 - c2 - d2;
            const float s1 = a2 + b2 + c2 + d2, s2 = std::sqrt(x * x + y * y);
            const float aniso = 1.f - std::sqrt((s1 + s2) / 2.f) / std::sqrt((s1 - s2) / 2.f);
            debugWrite(sv, PLT_DEBUG_VIEW_COHERENCE_ANISOTROPY, colourCode(kInferno, aniso));
        }
        propagate(beam, f3(cam.pos));
        if (cam.polarizer > 0.f) {
            const F3 W = normalize(f3(cam.w)), U = normalize(f3(cam.u));
            beam.rotateFrame(U, -W);
            const float pi = cam.polarizer;
            const float cth = std::cos(cam.polarizer_theta), sth = std::sin(cam.polarizer_theta);
            // (1 - p) I + p * MuellerPolarizer(theta), Mueller.slang:60-73
            const float P[4][4] = {{.5f * 1.f, .5f * cth, .5f * sth, 0.f}, {.5f * cth, .5f * (cth * cth), .5f * (cth * sth), 0.f},
                                   {.5f * sth, .5f * (cth * sth), .5f * (sth * sth), 0.f}, {0.f, 0.f, 0.f, 0.f}};
            for (int j = 0; j < beam.H; ++j) {
                const float in[4] = {beam.L[0][j], beam.L[1][j], beam.L[2][j], beam.L[3][j]};
                for (int r = 0; r < 4; ++r) {
                    float acc = 0.f;
                    for (int c = 0; c < 4; ++c) acc += ((1.f - pi) * (r == c ? 1.f : 0.f) + pi * P[r][c]) * in[c];
                    beam.L[r][j] = acc;
                }
            }
        }
        if (o.hwssMis) {
            float sum = 0.f;
            for (uint32_t j = 0; j < o.hwss; ++j) sum += beam.spdf[j];
            pathContribution *= sum > K_FLT_EPSILON ? beam.spdf[0] / sum : 0.f;
        } else {
            pathContribution *= 1.f / float(beam.H);
        }
        float Li[MAXH];
        for (int j = 0; j < beam.H; ++j) Li[j] = beam.L[0][j];
        const F3 rgb = spectrumToRgb(Li, beam.wl, (uint32_t)beam.H) * pathContribution;
        const F3 L = {std::max(0.f, rgb.x), std::max(0.f, rgb.y), std::max(0.f, rgb.z)};
        if (std::isfinite(L.x) && std::isfinite(L.y) && std::isfinite(L.z)) sv.Lrgb = sv.Lrgb + L;
        if (o.debugView) {
            // markDebug, pltpt_debug.slangh:31-50
            const F3& Ls = sv.Lrgb;
            if (std::isnan(Ls.x) || std::isnan(Ls.y) || std::isnan(Ls.z)) debugWrite(sv, PLT_DEBUG_VIEW_NANS, {5.f, 0.f, 3.f});
            if (std::isinf(Ls.x) || std::isinf(Ls.y) || std::isinf(Ls.z)) debugWrite(sv, PLT_DEBUG_VIEW_INFS, {2.f, 0.f, 5.f});
            debugWrite(sv, PLT_DEBUG_VIEW_PATH_LENGTH, colourCode(kMagma, (float)bounceIdx / float(o.maxBounces - 1)));
            debugWrite(sv, PLT_DEBUG_VIEW_HWSS_COMPS, colourCode(kMagma, (float)beam.H / float(o.hwss)));
            const float S0 = beam.L[0][0], S1 = beam.L[1][0], S2 = beam.L[2][0], S3 = beam.L[3][0];
            const float cp = std::sqrt(S3 * S3) / S0, lp = std::sqrt(S1 * S1 + S2 * S2) / S0;
            const float lpd = .5f * std::atan2(S2, S1);
            const float cl = std::cos(lpd), sl = std::sin(lpd);
            debugWrite(sv, PLT_DEBUG_VIEW_POLARIZATION, F3{lp * (cl * cl), cp, lp * (sl * sl)});
        }
    }

    // LightCollection's active triangles: flux > 0 (LightCollection.cpp:512-524)
    uint32_t activeCount() const {
        uint32_t n = 0;
        for (float f : s.lightFlux) n += f > 0.f ? 1u : 0u;
        return n;
    }
    uint32_t activeLight(uint32_t idx) const {
        for (uint32_t l = 0; l < (uint32_t)s.lightFlux.size(); ++l)
            if (s.lightFlux[l] > 0.f && idx-- == 0) return l;
        return kNone;
    }

    // getLightTypeSelectionProbabilities (LightSampling.slangh:40-55): env map, emissive geometry
    // (the scene's emissive lights when it has any), no analytic lights
    void typeProbabilities(float& pEnv, float& pEm, float& pAn) const {
        const bool useEnv = o.useEnv && s.env.present;
        const bool useEm = o.useEmissive && activeCount() > 0;
        const bool useAn = o.useAnalytic && !s.alights.empty();
        const float sum = (useEnv ? 1.f : 0.f) + (useEm ? 1.f : 0.f) + (useAn ? 1.f : 0.f);
        const float inv = sum > 0.f ? 1.f / sum : 0.f;
        pEnv = useEnv ? inv : 0.f;
        pEm = useEm ? inv : 0.f;
        pAn = useAn ? inv : 0.f;
    }

    // sampleLight for analytic lights (Rendering/Lights/LightHelpers.slang:71-289)
    bool sampleAnalytic(uint32_t li, F3 p, Solve& sv, F3& dir, float& dist, float* Li, float* wl, float& pdf) const {
        const plt_analytic_light& L = s.alights[li];
        const float* X = L.transform;
        const F3 ldirW = {L.dir[0], L.dir[1], L.dir[2]};
        if (L.type == PLT_LIGHT_POINT) {
            const F3 toLight = F3{L.pos[0], L.pos[1], L.pos[2]} - p;
            const float distSqr = std::max(dot(toLight, toLight), 1e-9f);
            dist = std::sqrt(distSqr);
            dir = toLight / dist;
            const float cosTheta = -dot(dir, ldirW);
            float falloff = 1.f;
            if (cosTheta < L.cos_opening_angle) {
                falloff = 0.f;
            } else if (L.penumbra_angle > 0.f) {
                const float delta = L.opening_angle - std::acos(cosTheta);
                const float t = std::min(std::max(delta / L.penumbra_angle, 0.f), 1.f);
                falloff = t * t * (3.f - 2.f * t);
            }
            sampleSpectrum(s, L.intensity_spectral_id, sv.wavelength, sv.sg, o.importanceSampleEmitters, o.hwss, Li, wl);
            for (uint32_t j = 0; j < o.hwss; ++j) Li[j] *= falloff / distSqr;
            pdf = 0.f;
            return true;
        }
        if (L.type == PLT_LIGHT_DIRECTIONAL) {
            dist = FLT_MAX;
            dir = -ldirW;
            sampleSpectrum(s, L.intensity_spectral_id, sv.wavelength, sv.sg, o.importanceSampleEmitters, o.hwss, Li, wl);
            pdf = 0.f;
            return true;
        }
        const float ux = sv.sg.next1D();
        const float uy = sv.sg.next1D();
        if (L.type == PLT_LIGHT_DISTANT) {
            const float z = ux * (1.f - L.cos_subtended_angle) + L.cos_subtended_angle;
            const float r = std::sqrt(1.f - z * z);
            const float phi = 6.28318530717958647693f * uy;
            const F3 d = {r * std::cos(phi), r * std::sin(phi), z};
            dir = normalize(F3{X[0] * d.x + X[1] * d.y + X[2] * d.z, X[4] * d.x + X[5] * d.y + X[6] * d.z, X[8] * d.x + X[9] * d.y + X[10] * d.z});
            dist = FLT_MAX;
            const float solidAngle = 6.28318530717958647693f * (1.f - L.cos_subtended_angle);
            sampleSpectrum(s, L.intensity_spectral_id, sv.wavelength, sv.sg, o.importanceSampleEmitters, o.hwss, Li, wl);
            pdf = 1.f / solidAngle;
            return true;
        }
        F3 lp;
        const float phi = 6.28318530717958647693f * uy;
        if (L.type == PLT_LIGHT_RECT) {
            lp = {ux * 2.f - 1.f, uy * 2.f - 1.f, 0.f};
        } else if (L.type == PLT_LIGHT_DISC) {
            const float r = std::sqrt(ux);
            lp = {r * std::cos(phi), r * std::sin(phi), 0.f};
        } else {
            const float ct = 1.0f - 2.0f * ux;
            const float st = std::sqrt(std::max(0.0f, 1.0f - ct * ct));
            lp = {st * std::cos(phi), st * std::sin(phi), ct};
        }
        const F3 posW = {X[0] * lp.x + X[1] * lp.y + X[2] * lp.z + X[3], X[4] * lp.x + X[5] * lp.y + X[6] * lp.z + X[7],
                         X[8] * lp.x + X[9] * lp.y + X[10] * lp.z + X[11]};
        const std::array<float, 9>& T = s.alightsIT[li];
        const F3 nl = L.type == PLT_LIGHT_SPHERE ? lp : F3{0.f, 0.f, 1.f};
        const F3 n = normalize(F3{T[0] * nl.x + T[1] * nl.y + T[2] * nl.z, T[3] * nl.x + T[4] * nl.y + T[5] * nl.z,
                                  T[6] * nl.x + T[7] * nl.y + T[8] * nl.z});
        const F3 toLight = posW - p;
        const float distSqr = std::max(dot(toLight, toLight), 1e-9f);
        dist = std::sqrt(distSqr);
        dir = toLight / dist;
        const float cosTheta = dot(n, -dir);
        if (cosTheta <= 0.f) return false;
        sampleSpectrum(s, L.intensity_spectral_id, sv.wavelength, sv.sg, o.importanceSampleEmitters, o.hwss, Li, wl);
        for (uint32_t j = 0; j < o.hwss; ++j) Li[j] *= L.surface_area * cosTheta / distSqr;
        pdf = distSqr / (cosTheta * L.surface_area);
        return true;
    }

    // evalTrianglePdf (EmissiveLightSamplerHelpers.slang:120-151) x triangle selection pdf
    // (EmissivePowerSampler.slang:90-122)
    float emissivePdf(F3 posW, uint32_t light, F3 hitPos, F3 hitNormal) const {
        if (light == kNone) return 0.f;
        const uint32_t na = o.uniformEmissive ? activeCount() : 0u;
        const float sel = o.uniformEmissive ? (na > 0 ? 1.f / (float)na : 0.f) : s.lightFlux[light] * s.invWeightsSum;
        const F3 toLight = hitPos - posW;
        const float distSqr = dot(toLight, toLight);
        if (distSqr <= FLT_MIN) return 0.f * sel;
        const F3 L = toLight / std::sqrt(distSqr);
        const float cosTheta = dot(hitNormal, -L);
        if (cosTheta <= 0.f) return 0.f * sel;
        const float denom = std::max(FLT_MIN, cosTheta * s.lightArea[light]);
        return sel * (distSqr / denom);
    }

    struct LightSample {
        bool analytic = false;
        float pdf = 0.f, distance = 0.f;
        F3 origin = {0.f, 0.f, 0.f}, dir = {0.f, 0.f, 0.f};
        Beam<float> beam;
    };

    // generateLightSample with the emissive sampler (LightSampling.slangh:108-206,
    // EmissivePowerSampler.slang:47-79, EmissiveLightSamplerHelpers.slang:56-118)
    bool generateLightSample(const ShadingData& sd, bool sampleRefl, bool sampleTrans, Solve& sv, LightSample& ls) const {
        ls = LightSample();
        ls.beam.H = (int)o.hwss;
        for (int c = 0; c < 4; ++c) for (int j = 0; j < MAXH; ++j) ls.beam.L[c][j] = 0.f;
        for (int j = 0; j < MAXH; ++j) { ls.beam.wl[j] = 0.f; ls.beam.spdf[j] = 1.f; }
        // selectLightType (LightSampling.slangh:40-84): the environment map and emissive geometry
        SampleGen& selSg = o.perTileSg ? sv.tilesg : sv.sg;
        float u = selSg.next1D();
        float pEnv, pEm, pAn;
        typeProbabilities(pEnv, pEm, pAn);
        float selectionPdf;
        bool envSel;
        if (u < pEnv) {
            envSel = true;
            selectionPdf = pEnv;
        } else {
            u -= pEnv;
            if (!(u < pEm)) {
                u -= pEm;
                if (!(u < pAn)) return false;
                // generateAnalyticLightSample (LightSampling.slangh:128-164)
                ls.analytic = true;
                const uint32_t n = (uint32_t)s.alights.size();
                const uint32_t li = std::min((uint32_t)(sv.sg.next1D() * (float)n), n - 1);
                const plt_analytic_light& AL = s.alights[li];
                float Li[MAXH], swl[MAXH], apdf;
                for (int j = 0; j < MAXH; ++j) { Li[j] = 0.f; swl[j] = 0.f; }
                F3 dir;
                float dist;
                if (!sampleAnalytic(li, sd.posW, sv, dir, dist, Li, swl, apdf)) return false;
                bool anyPos = false;
                for (uint32_t j = 0; j < o.hwss; ++j) {
                    Li[j] *= (float)n;
                    anyPos = anyPos || Li[j] > 0.f;
                }
                ls.pdf = apdf / (float)n;
                ls.origin = newRayOriginToward(sd, dir);
                ls.distance = dist;
                ls.dir = dir;
                if (AL.type == PLT_LIGHT_DIRECTIONAL || AL.type == PLT_LIGHT_DISTANT) {
                    const float omega = 4.f * 3.14159265358979323846f * (1.f - AL.cos_subtended_angle * AL.cos_subtended_angle);
                    ls.beam = sourceBeamDistant(-dir, omega, Li, swl, o.hwss, o.maxBeamOmega);
                } else {
                    ls.beam = sourceBeamArea(F3{AL.pos[0], AL.pos[1], AL.pos[2]}, -dir, AL.surface_area, dist, Li, swl, o.hwss, o.maxBeamOmega);
                }
                ls.pdf *= pAn;
                scaleBeam(ls.beam, 1.f / pAn);
                const bool isReflection = dot(sd.faceN, ls.dir) * dot(sd.faceN, sd.V) > 0.f;
                return anyPos && ls.pdf > 1e-6f && !(!sampleRefl && isReflection) && !(!sampleTrans && !isReflection);
            }
            envSel = false;
            selectionPdf = pEm;
        }
        if (envSel) {
            // generateEnvMapSample (LightSampling.slangh:86-104)
            const float u0 = sv.sg.next1D();
            const float u1 = sv.sg.next1D();
            float d[3], pdf;
            s.env.sample(u0, u1, d, pdf);
            float swl[MAXH], rad[3], L[MAXH];
            for (int j = 0; j < MAXH; ++j) { swl[j] = 0.f; L[j] = 0.f; }
            hwssWavelengths(sv.wavelength, o.hwss, swl);
            const F3 dir = f3(d);
            s.env.eval(d, rad);
            bool anyPos = false;
            for (uint32_t j = 0; j < o.hwss; ++j) {
                const float le = rgbToSpectrum(rad, swl[j]);
                L[j] = pdf > 0.f ? le / pdf : 0.f;
                anyPos = anyPos || L[j] > 0.f;
            }
            ls.beam = sourceBeamDistant(-dir, o.maxBeamOmega, L, swl, o.hwss, o.maxBeamOmega);
            ls.pdf = pdf;
            ls.origin = newRayOriginToward(sd, dir);
            ls.distance = FLT_MAX;
            ls.dir = dir;
            ls.pdf *= selectionPdf;
            scaleBeam(ls.beam, 1.f / selectionPdf);
            const bool isReflection = dot(sd.faceN, ls.dir) * dot(sd.faceN, sd.V) > 0.f;
            return anyPos && ls.pdf > 1e-6f && !(!sampleRefl && isReflection) && !(!sampleTrans && !isReflection);
        }
        bool valid = false;
        const uint32_t nl = (uint32_t)s.lightTri.size();
        if (nl > 0) {
            uint32_t ti;
            float triSelPdf;
            if (o.uniformEmissive) {
                // EmissiveUniformSampler.sampleLight (EmissiveUniformSampler.slang)
                const uint32_t na = activeCount();
                const float uLight = sv.sg.next1D();
                ti = activeLight(std::min((uint32_t)(uLight * (float)na), na - 1));
                triSelPdf = 1.f / (float)na;
            } else {
                // EmissivePowerSampler.sampleLight
                const float uLight = sv.sg.next1D();
                ti = std::min((uint32_t)(uLight * nl), nl - 1);
                const uint32_t px = s.alias[2 * (size_t)ti], py = s.alias[2 * (size_t)ti + 1];
                const float threshold = half_to_float((uint16_t)(px >> 16));
                const uint32_t selectAbove = ((px & 0xFFFFu) << 8u) | ((py >> 24u) & 0xFFu);
                const uint32_t selectBelow = py & 0xFFFFFFu;
                ti = (sv.sg.next1D() >= threshold) ? selectAbove : selectBelow;
                triSelPdf = s.lightFlux[ti] * s.invWeightsSum;
            }
            // sampleTriangle
            const float u0 = sv.sg.next1D(), u1 = sv.sg.next1D();
            const float su = std::sqrt(u0);
            const float bx = 1.f - su, by = u1 * su;
            const float bary[3] = {1.f - bx - by, bx, by};
            const float* P = &s.lightPos[9 * (size_t)ti];
            F3 tposW = f3(P) * bary[0];
            tposW = tposW + f3(P + 3) * bary[1];
            tposW = tposW + f3(P + 6) * bary[2];
            const F3 toL = tposW - sd.posW;
            const float distSqr = std::max(FLT_MIN, dot(toL, toL));
            const float tdist = std::sqrt(distSqr);
            const F3 tdir = toL / tdist;
            const F3 tn = f3(&s.lightNormal[3 * (size_t)ti]);
            const float cosTheta = dot(tn, -tdir);
            if (!(cosTheta <= 0.f)) {
                float Le[MAXH], swl[MAXH];
                for (int j = 0; j < MAXH; ++j) { Le[j] = 0.f; swl[j] = 0.f; }
                const Material<float>& lm = s.mats[s.triMat[s.lightTri[ti]]];
                sampleSpectrum(s, lm.emission, sv.wavelength, sv.sg, o.importanceSampleEmitters, o.hwss, Le, swl);
                const float white[3] = {1.f, 1.f, 1.f};
                for (uint32_t j = 0; j < o.hwss; ++j) Le[j] *= rgbToSpectrum(white, swl[j]);
                const float denom = std::max(FLT_MIN, cosTheta * s.lightArea[ti]);
                float tpdf = distSqr / denom;
                tpdf *= triSelPdf;
                // generateEmissiveSample
                float L[MAXH];
                bool anyPos = false;
                for (uint32_t j = 0; j < o.hwss; ++j) {
                    L[j] = tpdf > 0.f ? Le[j] / tpdf : 0.f;
                    anyPos = anyPos || L[j] > 0.f;
                }
                ls.pdf = tpdf;
                const float tp[3] = {tposW.x, tposW.y, tposW.z}, nn[3] = {tn.x, tn.y, tn.z};
                float lp[3];
                geom::computeRayOrigin(tp, nn, lp);
                const F3 lightPos = f3(lp);
                ls.origin = newRayOriginToward(sd, lightPos - sd.posW);
                const F3 toLight = lightPos - ls.origin;
                ls.distance = length(toLight);
                ls.dir = normalize(toLight);
                ls.beam = sourceBeamArea(tposW, -ls.dir, o.sourcingArea, ls.distance, L, swl, o.hwss, o.maxBeamOmega);
                valid = anyPos;
            }
        }
        ls.pdf *= selectionPdf;
        scaleBeam(ls.beam, 1.f / selectionPdf);
        const bool isReflection = dot(sd.faceN, ls.dir) * dot(sd.faceN, sd.V) > 0.f;
        return valid && ls.pdf > 1e-6f && !(!sampleRefl && isReflection) && !(!sampleTrans && !isReflection);
    }

    // closest-hit shadow ray, ShadowRays.slangh:96-135 (a hit needs dist > 0)
    bool shadowRay(F3 org, F3 dir, float tmin, float tmax, uint32_t& prim, float& t, float& b1, float& b2) const {
        const float O[3] = {org.x, org.y, org.z}, D[3] = {dir.x, dir.y, dir.z};
        prim = s.bvh.trace(O, D, tmin, tmax, false, t, b1, b2);
        return prim != kNone && t > 0.f;
    }
    uint32_t instanceOf(uint32_t prim) const { return s.triInst ? s.triInst[prim] : 0u; }

    // manifoldSampleVertex, Manifolds.slangh:84-108: sample a delta lobe towards the light
    bool manifoldSampleVertex(uint32_t prim, float b1, float b2, const ShadingData& sd, F3 lightDir, SampleGen& sg,
                              ManifoldSample& d) const {
        BSDFSample smp;
        if (!bsdfSampleHint(s, sd, sg, smp, d.wavelength, LOBE_DELTA, lightDir)) return false;
        d.pdf *= smp.pdf;
        d.hits[d.hitCount] = MSHit{prim, b1, b2, sd.posW, smp.lobe};
        d.dispersive = d.dispersive || (smp.lobe & (LOBE_DISPERSIVE_DELTA_REFLECTION | LOBE_DISPERSIVE_DELTA_TRANSMISSION)) != 0;
        ++d.hitCount;
        return true;
    }

    // traceMNEEOccluders, Manifolds.slangh:110-156
    bool traceMNEEOccluders(F3 rayO, F3 rayD, float tmin, float tmax, SampleGen& sg, int maxMS, ManifoldSample& d, Solve& sv) const {
        const F3 wi = -rayD;
        for (;;) {
            uint32_t prim;
            float t, b1, b2;
            ++sv.shadowRays;
            if (!shadowRay(rayO, rayD, tmin, tmax, prim, t, b1, b2)) return true;
            if (d.hitCount >= (int)o.mneeMaxOccluders || d.hitCount >= maxMS) return false;
            VertexData v = vertexData(s, prim, b1, b2);
            v.posW = rayO + rayD * t;
            const uint32_t mid = s.triMat[prim];
            const ShadingData sd = prepareShadingData(s, v, mid, wi);
            if (!(bsdfProps(s, mid).flags & PROP_MW_TRANSMISSIVE)) return false;
            if (!manifoldSampleVertex(prim, b1, b2, sd, -wi, sg, d) || (d.hits[d.hitCount - 1].lobe & LOBE_TRANSMISSION) == 0)
                return false;
            rayO = newRayOriginToward(sd, rayD);
            tmax -= t;
        }
    }

    // manifoldNEESample, Manifolds.slangh:171-281: Newton walk of the occluder chain on the
    // spherical-angle constraint, re-projected onto the same geometry instance by shadow rays,
    // then a visibility test from the last occluder to the light.
    bool manifoldNEESample(F3 visO, F3 visD, float visTmin, float visTmax, F3 origin, F3 lightPos, F3 lightDir, bool distant,
                           int maxMS, SampleGen& sg, ManifoldSample& d, Solve& sv) const {
        if (!traceMNEEOccluders(visO, visD, visTmin, visTmax, sg, maxMS, d, sv)) return false;
        if (d.hitCount == 0) return true;
        float beta[4] = {1.f, 1.f, 1.f, 1.f};
        bool success = false;
        while (!success) {
            success = true;
            for (int idx = 0; idx < d.hitCount; ++idx) {
                MSHit& h = d.hits[idx];
                const uint32_t mid = s.triMat[h.prim];
                const DSG g = differentialShadingGeometry(s, h.prim, h.b1, h.b2);
                const F3 p0 = idx == 0 ? origin : d.hits[idx - 1].posW;
                const F3pdv pdv0 = g.pdw(p0);
                const F3 p2 = idx + 1 == d.hitCount ? lightPos : d.hits[idx + 1].posW;
                F3pdv pdv2 = {lightDir, zero3(), zero3()};
                if (!distant) pdv2 = g.pdw(p2);
                const bool woIsIn = dot(pdv2.v, g.n.v) < 0.f;
                const F3pdv wi = woIsIn ? pdv0 : pdv2;
                const F3pdv wo = woIsIn ? pdv2 : pdv0;
                const F3kpdv wos = bsdfPartialDerivatives(s, mid, wi, g, h.lobe, d.wavelength);
                if (wos.v.x == 0.f && wos.v.y == 0.f && wos.v.z == 0.f) return false;
                float lenC;
                F3 stepDir;
                if (!manifoldOneStep(wo, wos, g.p, lenC, stepDir)) return false;
                if (lenC < o.mneeThreshold) continue;
                success = false;
                for (;;) {
                    if (++d.iterations > o.mneeMaxIterations) return false;
                    const F3 proposal = h.posW - stepDir * beta[idx];
                    F3 dirTo = proposal - p0;
                    const float dist = length(dirTo);
                    dirTo = dirTo / dist;
                    uint32_t prim;
                    float t, b1, b2;
                    ++sv.shadowRays;
                    const bool hit = shadowRay(p0, dirTo, std::max(1e-4f, .99f * dist), 1.01f * dist, prim, t, b1, b2);
                    if (!hit || instanceOf(h.prim) != instanceOf(prim)) {
                        beta[idx] /= 4.f;
                        continue;
                    }
                    h.prim = prim;
                    h.b1 = b1;
                    h.b2 = b2;
                    h.posW = p0 + dirTo * t;
                    beta[idx] = std::min(1.0f, 2.f * beta[idx]);
                    break;
                }
            }
        }
        const F3 pl = d.hits[d.hitCount - 1].posW;
        F3 dir;
        float dist;
        if (!distant) {
            dir = lightPos - pl;
            dist = length(dir);
            dir = dir / dist;
        } else {
            dir = lightDir;
            dist = FLT_MAX;
        }
        ++sv.shadowRays;
        const bool vis = visible(pl, dir, 1e-4f, dist);
        d.woLastHitToLight = dir;
        return vis;
    }

    // manifoldForwardUnwind, pltpt_solve.rt.slang:80-93
    void manifoldForwardUnwind(const ManifoldSample& ms, F3 origin, Beam<float>& beam, Solve& sv) const {
        for (int idx = ms.hitCount - 1; idx >= 0; --idx) {
            const MSHit& h = ms.hits[idx];
            VertexData v = vertexData(s, h.prim, h.b1, h.b2);
            v.posW = h.posW;
            const F3 p2 = idx == 0 ? origin : ms.hits[idx - 1].posW;
            const F3 wo = normalize(p2 - v.posW);
            forwardUnwindStep(h.prim, v, wo, h.lobe, beam, sv);
        }
    }

    // NEE, pltpt_solve.rt.slang:245-366
    void NEE(Solve& sv, int p, const Bounce* bounces, const ShadingData& sd, const VertexData& V, uint32_t mid) const {
        const Bounce& bounce = bounces[p];
        const Props props = bsdfProps(s, mid);
        const uint32_t lobes = props.lobes;
        const bool allowMSOnCurrentVertex =
            o.doMnee && p > 0 && (bounce.flags & FLAG_LAST_DELTA) == 0 && (props.flags & PROP_MW_REFLECTIVE) != 0;
        const bool sampleRefl = (lobes & 0x03u) != 0 || allowMSOnCurrentVertex;
        const bool sampleTrans = (lobes & 0x30u) != 0;
        if (!sampleRefl && !sampleTrans) return;
        LightSample ls;
        if (!generateLightSample(sd, sampleRefl, sampleTrans, sv, ls)) return;
        bool anyL = false;
        for (int j = 0; j < ls.beam.H; ++j) anyL = anyL || ls.beam.L[0][j] > 0.f;
        if (!anyL) return;
        if (!o.hwssMis && (bounce.flags & FLAG_DISPERSIVE)) ls.beam.H = 1;
        const bool doMis = o.doMis && !ls.analytic;   // pltpt_solve.rt.slang:276
        bool evalCurrentVertex = true;
        const int maxMSBounces = (int)o.maxBounces - p;
        if (!o.doMnee || maxMSBounces <= 0) {
            ++sv.shadowRays;
            if (!visible(ls.origin, ls.dir, 0.f, ls.distance)) return;
            if (doMis) scaleBeam(ls.beam, MISWeight(ls.pdf, bsdfPdf(s, sd, ls.dir, ls.beam.wl[0])));
        } else {
            const F3 lightDir = -ls.beam.r;
            float misBsdfPdf = 0.f;
            ManifoldSample ms;
            ms.wavelength = ls.beam.wl[0];
            const bool isReflection = dot(sd.N, lightDir) * dot(sd.N, sd.V) > 0.f;
            const bool currentVertexMS = isReflection && allowMSOnCurrentVertex;
            if (currentVertexMS) {
                if (!manifoldSampleVertex(bounce.prim, bounce.b1, bounce.b2, sd, lightDir, sv.sg, ms) ||
                    (ms.hits[0].lobe & LOBE_REFLECTION) == 0)
                    return;
            }
            const F3 origin = !currentVertexMS ? V.posW : sv.pathOrigin;
            const bool mneeOk = manifoldNEESample(ls.origin, ls.dir, 0.f, ls.distance, origin, ls.beam.posW, lightDir, ls.beam.distant,
                                                  maxMSBounces, sv.sg, ms, sv);
            if (o.debugView) {
                // MNEE views, pltpt_solve.rt.slang:319-325
                debugWrite(sv, PLT_DEBUG_VIEW_MNEE_ITERATIONS, colourCode(kInferno, ms.iterations / float(o.mneeMaxIterations)));
                if (ms.hitCount > 0 && mneeOk)
                    debugWrite(sv, PLT_DEBUG_VIEW_MNEE_BOUNCES, ms.hitCount == 1 ? F3{0.f, .3f, 1.f} : F3{1.f, 0.f, 0.f});
            }
            if (!mneeOk || ms.pdf < 1e-6f) return;
            if (ms.hitCount > 0) {
                if (!o.hwssMis && ms.dispersive) ls.beam.H = 1;
                if (!ls.beam.distant) {
                    ls.dir = ms.woLastHitToLight;
                    ls.beam.r = -ms.woLastHitToLight;
                    ls.beam.t = perp_stark(ls.beam.r);
                }
                scaleBeam(ls.beam, 1.f / ms.pdf);
                manifoldForwardUnwind(ms, origin, ls.beam, sv);
                if (currentVertexMS) {
                    evalCurrentVertex = false;
                    misBsdfPdf = bounce.lastNonDeltaPdf;
                }
            }
            if (doMis) {
                if (ms.hitCount == 0 || !currentVertexMS) misBsdfPdf = bsdfPdf(s, sd, ls.dir, ls.beam.wl[0]);
                scaleBeam(ls.beam, MISWeight(ls.pdf, misBsdfPdf * ms.pdf));
            }
        }
        // evalNEE, pltpt_solve.rt.slang:219-243
        if (evalCurrentVertex) {
            const ShadingData fsd = prepareShadingData(s, V, mid, -ls.beam.r);
            propagate(ls.beam, fsd.posW);
            const F3 wi = bounce.wi();
            bsdfEval(s, fsd, wi, LOBE_NON_DELTA, ls.beam);
            ++sv.unwindEvals;
            if (o.hwssMis) {
                float pdfs[MAXH];
                for (int j = 0; j < MAXH; ++j) pdfs[j] = 1.f;
                bsdfLambdaPdf(s, fsd, wi, LOBE_NON_DELTA, ls.beam, pdfs);
                for (uint32_t j = 0; j < o.hwss; ++j) ls.beam.spdf[j] *= pdfs[j];
            }
        }
        forwardUnwind(p, bounces, ls.beam, sv);
        measure(sv, p, bounce.pathContribution, ls.beam);
    }

    // evalEmissive, pltpt_solve.rt.slang:152-200
    void evalEmissive(Solve& sv, int p, const Bounce* bounces, const ShadingData& sd, uint32_t mid) const {
        const Bounce& bounce = bounces[p];
        const Props props = bsdfProps(s, mid);
        const bool didNEE = wasNEEAvailable(p, bounce.flags);
        if (!(o.useEmissive && (props.flags & PROP_EMISSIVE) && (o.doMis || !didNEE))) return;
        const bool needMIS = o.doMis && didNEE;
        const uint32_t light = s.primToLight[bounce.prim];
        const F3 hn = sd.frontFacing ? sd.faceN : -sd.faceN;
        float pEnv, pEm, pAn;
        typeProbabilities(pEnv, pEm, pAn);
        const float lightPdf = pEm * emissivePdf(sv.pathOrigin, light, sd.posW, hn);
        const float misWeight = needMIS ? MISWeight(bounce.lastNonDeltaPdf, lightPdf) : 1.f;
        float Le[MAXH], swl[MAXH];
        for (int j = 0; j < MAXH; ++j) { Le[j] = 0.f; swl[j] = 0.f; }
        sampleSpectrum(s, props.emissionId, sv.wavelength, sv.sg, o.importanceSampleEmitters, o.hwss, Le, swl);
        const float white[3] = {1.f, 1.f, 1.f};
        bool anyPos = false;
        for (uint32_t j = 0; j < o.hwss; ++j) {
            Le[j] *= misWeight * rgbToSpectrum(white, swl[j]);
            anyPos = anyPos || Le[j] > 0.f;
        }
        if (!anyPos) return;
        const float dist = length(sv.pathOrigin - sd.posW);
        Beam<float> beam = sourceBeamArea(sd.posW, bounce.wi(), o.sourcingArea, dist, Le, swl, o.hwss, o.maxBeamOmega);
        if (!o.hwssMis && (bounce.flags & FLAG_DISPERSIVE)) beam.H = 1;
        forwardUnwind(p, bounces, beam, sv);
        measure(sv, p, bounce.pathContribution, beam);
    }

    // onMiss, pltpt_solve.rt.slang:374-395
    void onMiss(Solve& sv, int p, const Bounce* bounces) const {
        const Bounce& bounce = bounces[p];
        const F3 wo = bounce.wi();
        const bool didNEE = wasNEEAvailable(p, bounce.flags);
        if (!(o.useEnv && s.env.present && (o.doMis || !didNEE))) return;
        const bool needMIS = o.doMis && didNEE;
        float pEnv, pEm, pAn;
        typeProbabilities(pEnv, pEm, pAn);
        const float nwo[3] = {-wo.x, -wo.y, -wo.z};
        const float lightPdf = pEnv * s.env.evalPdf(nwo);
        const float misWeight = needMIS ? MISWeight(bounce.lastNonDeltaPdf, lightPdf) : 1.f;
        float swl[MAXH], Le[MAXH], rad[3];
        for (int j = 0; j < MAXH; ++j) { swl[j] = 0.f; Le[j] = 0.f; }
        hwssWavelengths(sv.wavelength, o.hwss, swl);
        s.env.eval(nwo, rad);
        for (uint32_t j = 0; j < o.hwss; ++j) Le[j] = misWeight * rgbToSpectrum(rad, swl[j]);
        Beam<float> beam = sourceBeamDistant(wo, o.maxBeamOmega, Le, swl, o.hwss, o.maxBeamOmega);
        if (!o.hwssMis && (bounce.flags & FLAG_DISPERSIVE)) beam.H = 1;
        forwardUnwind(p, bounces, beam, sv);
        measure(sv, p, bounce.pathContribution, beam);
    }

    void solvePass(uint32_t px, uint32_t py, const Bounce* bounces, float* rgb, uint64_t* stats) const {
        const uint32_t tile = o.tileSize;
        Solve sv{SampleGen(px, py, frame, o.tinySg), SampleGen(px / tile, py / tile, frame << 2, o.tinySg)};
        sv.wavelength = sampleOneWavelength(sv.sg.next1D());
        sv.pathOrigin = f3(cam.pos);
        sv.pathNormal = normalize(f3(cam.w));
        for (int p = 0;; ++p) {
            const Bounce& b = bounces[p];
            if (b.flags & FLAG_MISS) {
                onMiss(sv, p, bounces);
                break;
            }
            const VertexData v = vertexData(s, b.prim, b.b1, b.b2);
            const uint32_t mid = s.triMat[b.prim];
            const ShadingData sd = prepareShadingData(s, v, mid, b.wi());
            if (o.doNee) NEE(sv, p, bounces, sd, v, mid);
            evalEmissive(sv, p, bounces, sd, mid);
            if (o.debugView && p == 0) {
                // geometry views (pltpt_solve.rt.slang:449-456); no texture coordinates, so uv = 0
                debugWrite(sv, PLT_DEBUG_VIEW_NORMALS, sd.N);
                debugWrite(sv, PLT_DEBUG_VIEW_UVS, F3{0.f, 0.f, 0.f});
            }
            if ((b.flags & FLAG_TERMINATED) || p == (int)o.maxBounces) break;
            sv.pathOrigin = v.posW;
            sv.pathNormal = sd.N;
        }
        if (o.debugView) {
            // lerp(colour, mean debug colour, intensity), pltpt_solve.rt.slang:470-475
            const float t = o.debugIntensity;
            const F3 dm = sv.dbg[3] > 0.f ? F3{sv.dbg[0], sv.dbg[1], sv.dbg[2]} / sv.dbg[3] : F3{0.f, 0.f, 0.f};
            sv.Lrgb = sv.Lrgb + (dm - sv.Lrgb) * t;
        }
        rgb[0] = sv.Lrgb.x;
        rgb[1] = sv.Lrgb.y;
        rgb[2] = sv.Lrgb.z;
        stats[0] += sv.shadowRays;
        stats[1] += sv.unwindEvals;
    }
};

}  // namespace

extern "C" {

// Scene for the path-tracing oracle (host arrays).
typedef struct plto_scene {
    uint32_t n_vertices, n_triangles, n_materials, n_profiles;
    const float* positions;              // [n_vertices][3]
    const float* normals;                // [n_vertices][3]
    const float* tangents;               // [n_vertices][4] or NULL
    const uint32_t* indices;             // [n_triangles][3]
    const uint32_t* tri_material;        // [n_triangles]
    const uint32_t* tri_instance;        // [n_triangles] geometry instance (mesh) of each triangle, or NULL
    const plt_material_record* materials;
    const plt_spectral_profile* profiles;
    const float* proposal_params;        // [11488] learned proposal parameters (learned_proposal renders), or NULL
    const struct plto_env* env;          // environment light, or NULL
    const plt_analytic_light* lights;    // analytic lights, or NULL
    uint32_t n_lights;
} plto_scene;

// Environment light: [height][width][3] linear RGB lat-long map, intensity, tint, Euler XYZ degrees.
typedef struct plto_env {
    const float* rgb;
    uint32_t width, height;
    float intensity, tint[3], rotation_deg[3];
} plto_env;

static bool loadEnv(const plto_env* e, plt_oracle_env::EnvMap& env) {
    if (!e) return true;
    if (!e->rgb || e->width == 0 || e->height == 0) return false;
    env.width = e->width;
    env.height = e->height;
    env.rgb.assign(e->rgb, e->rgb + 3 * (size_t)e->width * e->height);
    for (int k = 0; k < 3; ++k) env.scale[k] = e->intensity * e->tint[k];
    env.setRotation(e->rotation_deg);
    env.buildImportance();
    env.present = true;
    return true;
}

// The sampler on given inputs: out[12 i ..] as plt_env_map_query (sampled direction, pdf, eval,
// evalPdf; eval and evalPdf of dirs[i], zeros when dirs is NULL).
int plto_env_query(const plto_env* e, const float* u, const float* dirs, uint32_t n, float* out) {
    plt_oracle_env::EnvMap env;
    if (!e || !loadEnv(e, env)) return PLT_INVALID_ARG;
    for (uint32_t i = 0; i < n; ++i) {
        float d[3], pdf, c[3];
        env.sample(u[2 * (size_t)i], u[2 * (size_t)i + 1], d, pdf);
        env.eval(d, c);
        float* o = out + 12 * (size_t)i;
        o[0] = d[0]; o[1] = d[1]; o[2] = d[2]; o[3] = pdf;
        o[4] = c[0]; o[5] = c[1]; o[6] = c[2]; o[7] = env.evalPdf(d);
        if (dirs) {
            const float* q = dirs + 3 * (size_t)i;
            env.eval(q, c);
            o[8] = c[0]; o[9] = c[1]; o[10] = c[2]; o[11] = env.evalPdf(q);
        } else {
            o[8] = o[9] = o[10] = o[11] = 0.f;
        }
    }
    return PLT_OK;
}

// Renders frames frame .. frame + frames - 1 of a width x height image into rgb [height][width][3]
// (their mean).  Optional per-path records [height*width][max_bounces+1] of bounce primitive
// (0xFFFFFFFF when absent), lobe and flags, of the last frame.
// stats (optional, 3 values): paths, shadow rays, forward BSDF evaluations.
int plto_render(const plto_scene* sc, const plt_camera* cam, const plt_options* opt, uint32_t width, uint32_t height,
                uint32_t frame, uint32_t frames, int threads, float* rgb, uint32_t* rec_prim, uint32_t* rec_lobe,
                uint32_t* rec_flags, uint64_t* stats) {
    if (frames == 0) return PLT_INVALID_ARG;
    if (!sc || !cam || !opt || !rgb) return PLT_INVALID_ARG;
    if (opt->hwss < 1 || (opt->hwss > 4 && opt->hwss != 8) || opt->mnee_max_occluders > 4) return PLT_NOT_SUPPORTED;
    Scene s;
    s.nv = sc->n_vertices;
    s.nt = sc->n_triangles;
    s.pos = sc->positions;
    s.nrm = sc->normals;
    s.tan = sc->tangents;
    s.idx = sc->indices;
    s.triMat = sc->tri_material;
    s.triInst = sc->tri_instance;
    s.tables.profiles = sc->profiles;
    s.tables.count = sc->n_profiles;
    s.mats.reserve(sc->n_materials);
    for (uint32_t i = 0; i < sc->n_materials; ++i) {
        s.mats.push_back(decodeMaterial<float>(sc->materials[i]));
        s.matFlags.push_back(recordDoubleSided(sc->materials[i]) ? 1u : 0u);
    }
    for (uint32_t t = 0; t < s.nt; ++t)
        if (s.triMat[t] >= sc->n_materials) return PLT_BAD_MATERIAL;
    s.triVerts.resize(9 * (size_t)s.nt);
    for (uint32_t t = 0; t < s.nt; ++t)
        for (int k = 0; k < 3; ++k)
            for (int c = 0; c < 3; ++c) s.triVerts[9 * (size_t)t + 3 * k + c] = s.pos[3 * (size_t)s.idx[3 * (size_t)t + k] + c];
    buildLights(s);
    s.bvh.build(s.triVerts.data(), s.nt);

    Options o;
    o.maxBounces = opt->max_bounces;
    o.tileSize = opt->tile_size ? opt->tile_size : 512;
    o.hwss = opt->hwss;
    o.hwssMis = opt->hwss_do_mis != 0;
    o.useDirect = opt->use_direct_light != 0;
    o.useEmissive = opt->use_emissive_lights != 0;
    o.doNee = opt->do_nee != 0;
    o.doMis = opt->do_nee != 0 && opt->do_mis != 0;
    o.doRR = opt->do_russian_roulette != 0;
    o.perTileSg = opt->do_nee != 0 && opt->nee_use_per_tile_sg != 0;
    o.importanceSampleEmitters = opt->do_importance_sample_emitters != 0;
    o.sourcingArea = opt->sourcing_area_from_emissive_geometry;
    o.maxBeamOmega = opt->sourcing_max_beam_omega;
    o.doMnee = opt->do_nee != 0 && opt->do_mnee != 0;
    o.mneeMaxOccluders = std::min<uint32_t>(opt->mnee_max_occluders, 4u);
    o.mneeMaxIterations = opt->mnee_max_iterations;
    o.mneeThreshold = opt->mnee_solver_threshold;
    o.learned = opt->learned_proposal != 0;
    o.learnedProb = opt->learned_proposal_prob;
    o.useEnv = opt->use_env_light != 0;
    o.useAnalytic = opt->use_analytic_lights != 0;
    o.uniformEmissive = opt->emissive_sampler == 0;
    o.alphaMask = opt->alpha_masking != 0;
    o.tinySg = opt->sample_generator == PLT_SAMPLE_GENERATOR_TINY_UNIFORM;
    o.debugView = opt->debug_view;
    o.debugIntensity = opt->debug_view_intensity;
    for (uint32_t i = 0; i < sc->n_lights; ++i) {
        const plt_analytic_light& l = sc->lights[i];
        s.alights.push_back(l);
        const float* t = l.transform;
        const double a[9] = {t[0], t[1], t[2], t[4], t[5], t[6], t[8], t[9], t[10]};
        const double cof[9] = {a[4] * a[8] - a[5] * a[7], a[5] * a[6] - a[3] * a[8], a[3] * a[7] - a[4] * a[6],
                               a[2] * a[7] - a[1] * a[8], a[0] * a[8] - a[2] * a[6], a[1] * a[6] - a[0] * a[7],
                               a[1] * a[5] - a[2] * a[4], a[2] * a[3] - a[0] * a[5], a[0] * a[4] - a[1] * a[3]};
        const double det = a[0] * cof[0] + a[1] * cof[1] + a[2] * cof[2];
        std::array<float, 9> it{};
        for (int k = 0; k < 9; ++k) it[k] = det != 0.0 ? (float)(cof[k] / det) : 0.f;
        s.alightsIT.push_back(it);
    }
    if (!loadEnv(sc->env, s.env)) return PLT_INVALID_ARG;
    if (o.learned) {
        if (!sc->proposal_params || !(o.learnedProb > 0.f && o.learnedProb < 1.f)) return PLT_INVALID_ARG;
        s.net.reset(new plt_oracle_mlp::Net(sc->proposal_params, true));
        s.matFeat.resize(4 * (size_t)sc->n_materials);
        for (uint32_t i = 0; i < sc->n_materials; ++i) proposalFeatures(s.mats[i], s.tables, &s.matFeat[4 * (size_t)i]);
    }

    const uint32_t nb = o.maxBounces + 1;
    const int64_t npix = (int64_t)width * height;
    uint64_t shadow = 0, evals = 0;
    std::vector<double> acc(frames > 1 ? 3 * (size_t)npix : 0, 0.0);
    for (uint32_t f = 0; f < frames; ++f) {
    Renderer R{s, *cam, o, width, height, frame + f};
#ifdef _OPENMP
#pragma omp parallel num_threads(threads > 0 ? threads : 1) if (threads != 1) reduction(+ : shadow, evals)
#endif
    {
        std::vector<Bounce> bounces(nb);
        uint64_t st[2] = {0, 0};
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 16)
#endif
        for (int64_t i = 0; i < npix; ++i) {
            const uint32_t px = (uint32_t)(i % width), py = (uint32_t)(i / width);
            for (uint32_t b = 0; b < nb; ++b) bounces[b] = Bounce();
            R.samplePass(px, py, bounces.data());
            R.solvePass(px, py, bounces.data(), rgb + 3 * i, st);
            if (rec_prim || rec_lobe || rec_flags) {
                for (uint32_t b = 0; b < nb; ++b) {
                    if (rec_prim) rec_prim[i * nb + b] = bounces[b].prim;
                    if (rec_lobe) rec_lobe[i * nb + b] = bounces[b].lobe;
                    if (rec_flags) rec_flags[i * nb + b] = bounces[b].flags;
                }
            }
        }
        shadow += st[0];
        evals += st[1];
    }
    if (frames > 1) for (size_t k = 0; k < acc.size(); ++k) acc[k] += rgb[k];
    }
    if (frames > 1) for (size_t k = 0; k < acc.size(); ++k) rgb[k] = (float)(acc[k] / frames);
    if (stats) {
        stats[0] = (uint64_t)npix;
        stats[1] = shadow;
        stats[2] = evals;
    }
    return PLT_OK;
}

// The light collection's alias table as the oracle builds it (for the library's table check):
// returns the light-triangle count; alias [2*count] (may be NULL to query), inv_weight_sum.
uint32_t plto_light_table(const plto_scene* sc, uint32_t* alias_out, uint32_t* light_tri_out, float* inv_weight_sum) {
    Scene s;
    s.nt = sc->n_triangles;
    s.pos = sc->positions;
    s.idx = sc->indices;
    s.triMat = sc->tri_material;
    s.tables.profiles = sc->profiles;
    s.tables.count = sc->n_profiles;
    for (uint32_t i = 0; i < sc->n_materials; ++i) s.mats.push_back(decodeMaterial<float>(sc->materials[i]));
    buildLights(s);
    const uint32_t nl = (uint32_t)s.lightTri.size();
    if (alias_out) std::memcpy(alias_out, s.alias.data(), 8 * (size_t)nl);
    if (light_tri_out) std::memcpy(light_tri_out, s.lightTri.data(), 4 * (size_t)nl);
    if (inv_weight_sum) *inv_weight_sum = s.invWeightsSum;
    return nl;
}

}  // extern "C"
