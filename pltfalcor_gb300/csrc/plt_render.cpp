// Host side of the PLTPT render pass: per-material property words, the emissive-triangle light
// collection with the power sampler's alias table, render-buffer management and the frame loop.
// Paths cited are inside ssteinberg/PLTFalcor.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "plt_context.h"

namespace {

plt_status cudaFail(plt_context* ctx, cudaError_t e) {
    if (ctx) ctx->lastCudaError = (int)e;
    return e == cudaErrorMemoryAllocation ? PLT_OOM : PLT_CUDA_ERROR;
}
#define PLT_CUDA(ctx, call)                               \
    do {                                                  \
        cudaError_t e_ = (call);                          \
        if (e_ != cudaSuccess) return cudaFail(ctx, e_);  \
    } while (0)

template <class T> plt_status upload(plt_context* ctx, T*& dst, const T* src, size_t count) {
    cudaFree(dst);
    dst = nullptr;
    if (count == 0) return PLT_OK;
    PLT_CUDA(ctx, cudaMalloc(&dst, sizeof(T) * count));
    PLT_CUDA(ctx, cudaMemcpy(dst, src, sizeof(T) * count, cudaMemcpyHostToDevice));
    return PLT_OK;
}

struct V3 { float x, y, z; };
V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 crossv(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
float lengthv(V3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

// snorm16 octahedral encode -> decode of a unit normal, the storage of the emissive triangles'
// face normals (encodeNormal2x16 / decodeNormal2x16, Utils/Math/PackedFormats.slang:50-62,
// FormatConversion.slang:216-258, MathHelpers.slang:147-185)
void octWrap(float& x, float& y) {
    const float nx = (1.f - std::fabs(y)) * (x >= 0.f ? 1.f : -1.f);
    const float ny = (1.f - std::fabs(x)) * (y >= 0.f ? 1.f : -1.f);
    x = nx;
    y = ny;
}
int32_t toSnorm16(float v) {
    v = std::isnan(v) ? 0.f : std::fmin(std::fmax(v, -1.f), 1.f);
    return (int32_t)std::trunc(v * 32767.f + (v >= 0.f ? 0.5f : -0.5f));
}
V3 storedNormal(V3 n) {
    const float s = 1.f / (std::fabs(n.x) + std::fabs(n.y) + std::fabs(n.z));
    float px = n.x * s, py = n.y * s;
    if (n.z < 0.f) octWrap(px, py);
    const uint32_t packed = ((uint32_t)toSnorm16(px) & 0xFFFFu) | ((uint32_t)toSnorm16(py) << 16);
    const int32_t bx = (int32_t)(packed << 16) >> 16, by = (int32_t)packed >> 16;
    float x = std::fmax((float)bx / 32767.f, -1.f), y = std::fmax((float)by / 32767.f, -1.f);
    const float z = 1.f - std::fabs(x) - std::fabs(y);
    if (z < 0.f) octWrap(x, y);
    const float l = std::sqrt(x * x + y * y + z * z);
    return {x / l, y / l, z / l};
}

// binary16 of a threshold in [0, 1], round to nearest even
uint16_t halfBits(float f) {
    uint32_t x;
    std::memcpy(&x, &f, 4);
    const uint32_t sign = (x >> 16) & 0x8000u;
    const int32_t e = (int32_t)((x >> 23) & 0xFF) - 127 + 15;
    uint32_t m = x & 0x7FFFFFu;
    if (((x >> 23) & 0xFF) == 0xFF) return (uint16_t)(sign | 0x7C00u | (m ? 0x200u : 0u));
    if (e >= 31) return (uint16_t)(sign | 0x7C00u);
    if (e <= 0) {
        if (e < -10) return (uint16_t)sign;
        m |= 0x800000u;
        const int shift = 14 - e;
        uint32_t hm = m >> shift;
        const uint32_t rem = m & ((1u << shift) - 1u), half = 1u << (shift - 1);
        if (rem > half || (rem == half && (hm & 1u))) ++hm;
        return (uint16_t)(sign | hm);
    }
    uint32_t h = ((uint32_t)e << 10) | (m >> 13);
    const uint32_t rem = m & 0x1FFFu;
    if (rem > 0x1000u || (rem == 0x1000u && (h & 1u))) ++h;
    return (uint16_t)(sign | h);
}

// Alias table over the light weights, EmissivePowerSampler::generateAliasTable
// (Rendering/Lights/EmissivePowerSampler.cpp:86-175): weights scaled to mean 1 and ordered
// small to large (a stable order for equal weights), paired head/tail, entries shuffled with a
// default-seeded mt19937 (full-range draws), packed as {binary16 threshold | alias >> 8,
// alias & 0xFF << 24 | own index}.
void buildAliasTable(const std::vector<float>& flux, std::vector<uint2>& table, float& invWeightsSum) {
    const uint32_t N = (uint32_t)flux.size();
    table.assign(N, make_uint2(0u, 0u));
    if (N == 0) { invWeightsSum = 0.f; return; }
    std::vector<float> w(flux);
    double sum = 0.0;
    for (float f : w) sum += f;
    for (float& f : w) f *= N / float(sum);
    std::vector<uint32_t> perm(N);
    for (uint32_t i = 0; i < N; ++i) perm[i] = i;
    std::stable_sort(perm.begin(), perm.end(), [&](uint32_t a, uint32_t b) { return w[a] < w[b]; });
    std::vector<float> thr(N, 0.f);
    std::vector<uint32_t> alias(N, 0u);
    uint32_t head = 0, tail = N - 1;
    while (head != tail) {
        const uint32_t i = perm[head], j = perm[tail];
        thr[i] = w[i];
        alias[i] = j;
        w[j] -= 1.0f - w[i];
        if (head == tail - 1) {
            thr[j] = 1.0f;
            alias[j] = j;
            break;
        }
        if (w[j] < 1.0f) {
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
        std::swap(alias[i], alias[dst]);
        std::swap(perm[i], perm[dst]);
    }
    for (uint32_t i = 0; i < N; ++i) {
        const uint32_t prob = (uint32_t)halfBits(thr[i]) << 16u;
        const uint32_t a = alias[i] & 0xFFFFFFu, own = perm[i] & 0xFFFFFFu;
        table[i] = make_uint2(prob | ((a >> 8u) & 0xFFFFu), ((a & 0xFFu) << 24u) | own);
    }
    invWeightsSum = 1.0f / float(sum);
}

// Emissive triangles (materials with an emission profile, in primitive order), their face normal
// and area (computeFaceNormalAndAreaW, Scene/Scene.slang:482-497) and luminous flux
// luminance(profile rgb) * area * pi (Scene/Lights/FinalizeIntegration.cs.slang:60-110).
plt_status buildLights(plt_context* ctx) {
    const uint32_t nt = ctx->nTris;
    std::vector<uint32_t> primToLight(nt, 0xFFFFFFFFu), lightTri;
    for (uint32_t t = 0; t < nt; ++t) {
        const uint32_t m = ctx->hTriMat[t];
        if (m >= ctx->hMats.size()) return PLT_BAD_MATERIAL;
        const plt_material_record& r = ctx->hMats[m];
        if (r.type != PLT_MATERIAL_DIFFUSE || r.emission_spectral_id == PLT_NO_SPECTRAL_PROFILE) continue;
        primToLight[t] = (uint32_t)lightTri.size();
        lightTri.push_back(t);
    }
    const uint32_t nl = (uint32_t)lightTri.size();
    std::vector<float> pos(9 * (size_t)nl), nrm(3 * (size_t)nl), area(nl), flux(nl);
    std::vector<uint32_t> emission(nl);
    for (uint32_t l = 0; l < nl; ++l) {
        const uint32_t t = lightTri[l];
        V3 p[3];
        for (int k = 0; k < 3; ++k) {
            const float* v = &ctx->hPos[3 * (size_t)ctx->hIdx[3 * (size_t)t + k]];
            p[k] = {v[0], v[1], v[2]};
            std::memcpy(&pos[9 * (size_t)l + 3 * k], v, 12);
        }
        const V3 N = crossv(sub(p[1], p[0]), sub(p[2], p[0]));
        const float len = lengthv(N);
        const V3 n = storedNormal({N.x / len, N.y / len, N.z / len});
        nrm[3 * (size_t)l] = n.x;
        nrm[3 * (size_t)l + 1] = n.y;
        nrm[3 * (size_t)l + 2] = n.z;
        area[l] = 0.5f * len;
        const uint32_t em = ctx->hMats[ctx->hTriMat[t]].emission_spectral_id;
        emission[l] = em;
        float rgb[3] = {0.f, 0.f, 0.f};
        if (em < ctx->hProfiles.size())
            for (int c = 0; c < 3; ++c) rgb[c] = std::max(0.f, ctx->hProfiles[em].rgb[c]);
        const float lum = rgb[0] * 0.2126f + rgb[1] * 0.7152f + rgb[2] * 0.0722f;
        flux[l] = lum * area[l] * 3.14159265358979323846f;
    }
    std::vector<uint2> table;
    buildAliasTable(flux, table, ctx->invWeightsSum);
    plt_status s;
    if ((s = upload(ctx, ctx->dLightPos, pos.data(), pos.size())) != PLT_OK) return s;
    if ((s = upload(ctx, ctx->dLightNrm, nrm.data(), nrm.size())) != PLT_OK) return s;
    if ((s = upload(ctx, ctx->dLightArea, area.data(), area.size())) != PLT_OK) return s;
    if ((s = upload(ctx, ctx->dLightFlux, flux.data(), flux.size())) != PLT_OK) return s;
    if ((s = upload(ctx, ctx->dAlias, table.data(), table.size())) != PLT_OK) return s;
    if ((s = upload(ctx, ctx->dLightEmission, emission.data(), emission.size())) != PLT_OK) return s;
    if ((s = upload(ctx, ctx->dPrimToLight, primToLight.data(), primToLight.size())) != PLT_OK) return s;
    ctx->nLights = nl;
    return PLT_OK;
}

// Render buffers for npix paths and maxB bounces: path state, queues, bounce buffer, accumulator.
plt_status ensureRenderBuffers(plt_context* ctx, uint32_t npix, uint32_t maxB) {
    if (ctx->dPt && ctx->ptNpix == npix && ctx->ptMaxB == maxB) return PLT_OK;
    cudaFree(ctx->dPt);
    ctx->dPt = nullptr;
    ctx->ptBytes = 0;
    const size_t n = npix, nb = (size_t)maxB + 1;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    const size_t pathBytes = al(4 * n * 4) + 2 * al(3 * n * 4) + 5 * al(n * 4) + 2 * al(n * 4) + 2 * al(n * 4) + al((nb + 2) * 4);
    const size_t bounceBytes = 2 * al(nb * n * 4) * 2 + 5 * al(nb * n * 4);
    const size_t accumBytes = al(3 * n * 8);
    const size_t total = pathBytes + bounceBytes + accumBytes;
    PLT_CUDA(ctx, cudaMalloc(&ctx->dPt, total));
    ctx->ptBytes = total;
    char* p = static_cast<char*>(ctx->dPt);
    auto take = [&](size_t bytes) { void* r = p; p += al(bytes); return r; };
    plt::PtParams& P = ctx->pt;
    P.sg = (uint32_t*)take(4 * n * 4);
    P.org = (float*)take(3 * n * 4);
    P.dir = (float*)take(3 * n * 4);
    P.wl = (float*)take(n * 4);
    P.weight = (float*)take(n * 4);
    P.pdf = (float*)take(n * 4);
    P.thp = (float*)take(n * 4);
    P.lndp = (float*)take(n * 4);
    P.pflags = (uint32_t*)take(n * 4);
    P.plen = (uint32_t*)take(n * 4);
    P.queue0 = (uint32_t*)take(n * 4);
    P.queue1 = (uint32_t*)take(n * 4);
    P.qcount = (uint32_t*)take((nb + 2) * 4);   // per-segment queue lengths + the manifold-walk task count
    P.mneeCount = P.qcount + nb + 1;
    P.bBary = (float*)take(2 * nb * n * 4);
    P.bEw = (float*)take(2 * nb * n * 4);
    P.bPrim = (uint32_t*)take(nb * n * 4);
    P.bLobe = (uint32_t*)take(nb * n * 4);
    P.bFlags = (uint32_t*)take(nb * n * 4);
    P.bContrib = (float*)take(nb * n * 4);
    P.bLndp = (float*)take(nb * n * 4);
    P.accum = (double*)take(3 * n * 8);
    ctx->ptNpix = npix;
    ctx->ptMaxB = maxB;
    return PLT_OK;
}

}  // namespace

namespace plt {
cudaError_t launchResolve(const double* accum, uint32_t npix, uint32_t frames, float* out, int numSMs, cudaStream_t stream);
}

// getProperties / getLobes of the PLT*BSDF.slang wrappers, double-sidedness
// (BasicMaterial::adjustDoubleSidedFlag, BasicMaterial.cpp:719-731) and the alpha-mask test.
uint2 pltMaterialProps(const plt_material_record& r, const pltdev::DevMaterial& d) {
    constexpr float kQcut = .15f;   // QcutoffForMS, IMaterialInstance.slang:44
    uint32_t flags = 0, lobes = 0;
    auto rough = [](float q) { return q == 0.f ? 0x04u : 0x06u; };
    switch (r.type) {
    case PLT_MATERIAL_DIFFUSE:
        flags = r.emission_spectral_id != PLT_NO_SPECTRAL_PROFILE ? plt::kPropEmissive : 0u;
        lobes = 0x01u;
        break;
    case PLT_MATERIAL_DIELECTRIC: {
        const float q = d.p[pltdev::PG_Q];
        flags = plt::kPropTransmissive | (q < kQcut ? plt::kPropMwTransmissive : 0u);
        const uint32_t dt = d.p[pltdev::PG_B] != 0.f ? 0x80u : 0x40u;
        lobes = q == 0.f ? (0x04u | dt) : (0x04u | dt | 0x02u | 0x20u);
        break;
    }
    case PLT_MATERIAL_CONDUCTOR:
    case PLT_MATERIAL_OPAQUE_DIELECTRIC:
    case PLT_MATERIAL_COATED_CONDUCTOR:
    case PLT_MATERIAL_COATED_OPAQUE_DIELECTRIC: {
        const float q = d.p[pltdev::PF_Q];
        flags = q < kQcut ? plt::kPropMwReflective : 0u;
        lobes = rough(q);
        break;
    }
    case PLT_MATERIAL_GRATED_CONDUCTOR:
    case PLT_MATERIAL_GRATED_OPAQUE_DIELECTRIC:
        flags = plt::kPropMwReflective;
        lobes = rough(d.p[pltdev::PF_Q]) | 0x08u;
        break;
    case PLT_MATERIAL_THIN_DIELECTRIC:
        flags = plt::kPropTransmissive | plt::kPropMwReflective | plt::kPropMwTransmissive;
        lobes = 0x04u | 0x40u;
        break;
    case PLT_MATERIAL_MULTILAYERED_STACK:
        flags = plt::kPropMwReflective;
        lobes = 0x04u;
        break;
    default: break;
    }
    const bool dsided = (r.flags & PLT_MATERIAL_FLAG_DOUBLE_SIDED) != 0 || plt::halfToFloat(r.specular_transmission) > 0.f ||
                        plt::halfToFloat(r.diffuse_transmission) > 0.f;
    const bool alphaZero = plt::halfToFloat(r.base_color[3]) == 0.f;
    return make_uint2(flags | (lobes << 8) | (dsided ? plt::kPropDoubleSided : 0u) | (alphaZero ? plt::kPropAlphaZero : 0u),
                      r.emission_spectral_id);
}

void pltReleaseRenderState(plt_context* ctx) {
    void* ptrs[] = {ctx->dProfileIcdf, ctx->dMatProps, ctx->dPos, ctx->dIdx, ctx->dNrm, ctx->dTan, ctx->dTriInst, ctx->dLightPos, ctx->dLightNrm,
                    ctx->dLightArea, ctx->dLightFlux, ctx->dAlias, ctx->dPrimToLight, ctx->dLightEmission, ctx->dPt, ctx->dPtStats, ctx->dPtMix, ctx->dMneeTasks};
    for (void* p : ptrs) cudaFree(p);
}

extern "C" {

plt_status plt_set_scene_shading(plt_context* ctx, const float* normals, const float* tangents, uint32_t n_vertices,
                                 const uint32_t* tri_instance) {
    if (!ctx || !normals) return PLT_INVALID_ARG;
    if (n_vertices != ctx->nVerts || ctx->nTris == 0) return PLT_INVALID_ARG;
    for (size_t i = 0; i < 3 * (size_t)n_vertices; ++i)
        if (!std::isfinite(normals[i])) return PLT_NAN_INPUT;
    plt_status s;
    if ((s = upload(ctx, ctx->dNrm, normals, 3 * (size_t)n_vertices)) != PLT_OK) return s;
    cudaFree(ctx->dTan);
    ctx->dTan = nullptr;
    if (tangents && (s = upload(ctx, ctx->dTan, tangents, 4 * (size_t)n_vertices)) != PLT_OK) return s;
    {
        std::vector<uint32_t> inst(ctx->nTris, 0u);
        if (tri_instance) std::memcpy(inst.data(), tri_instance, sizeof(uint32_t) * ctx->nTris);
        if ((s = upload(ctx, ctx->dTriInst, inst.data(), inst.size())) != PLT_OK) return s;
    }
    if ((s = buildLights(ctx)) != PLT_OK) return s;
    ctx->shadingReady = true;
    return PLT_OK;
}

plt_status plt_render(plt_context* ctx, const plt_camera* camera, uint32_t width, uint32_t height, uint32_t frame_begin,
                      uint32_t frame_count, float* out_rgba, void* stream) {
    if (!ctx || !camera || !out_rgba || frame_count == 0) return PLT_INVALID_ARG;
    if (((uintptr_t)out_rgba & 15u) != 0) return PLT_INVALID_ARG;
    if (!ctx->shadingReady || ctx->nTris == 0 || ctx->nMats == 0) return PLT_INVALID_ARG;
    const plt_options& o = ctx->opt;
    if (o.hwss < 1 || o.hwss > 4) return PLT_NOT_SUPPORTED;
    if (o.mnee_max_occluders > 4) return PLT_NOT_SUPPORTED;
    if (o.max_bounces > 64) return PLT_NOT_SUPPORTED;
    const bool learned = o.learned_proposal != 0;
    if (learned && (!ctx->propReady || !ctx->dMatFeat || !(o.learned_proposal_prob > 0.f && o.learned_proposal_prob < 1.f)))
        return PLT_INVALID_ARG;
    const uint64_t npix64 = (uint64_t)width * height;
    if (npix64 == 0) return PLT_OK;
    if (npix64 > (1u << 26)) return PLT_NOT_SUPPORTED;
    const uint32_t npix = (uint32_t)npix64;
    plt_status s = ensureRenderBuffers(ctx, npix, o.max_bounces);
    if (s != PLT_OK) return s;
    // path state of learned renders: the product of primary-sample MIS densities per path
    const size_t mixBytes = learned ? (size_t)npix * sizeof(float) : 0;
    if (learned && ctx->ptMixBytes < mixBytes) {
        cudaFree(ctx->dPtMix);
        ctx->dPtMix = nullptr;
        ctx->ptMixBytes = 0;
        PLT_CUDA(ctx, cudaMalloc(&ctx->dPtMix, mixBytes));
        ctx->ptMixBytes = mixBytes;
    }
    if (!ctx->dPtStats) PLT_CUDA(ctx, cudaMalloc(&ctx->dPtStats, 4 * sizeof(unsigned long long)));
    const cudaStream_t st = (cudaStream_t)stream;
    plt::PtParams& P = ctx->pt;
    P.nodes = ctx->dNodes;
    P.tris = ctx->dTris;
    P.pos = ctx->dPos;
    P.nrm = ctx->dNrm;
    P.tan = ctx->dTan;
    P.idx = ctx->dIdx;
    P.triMat = ctx->dTriMaterial;
    P.triInst = ctx->dTriInst;
    P.nTris = ctx->nTris;
    P.mats = ctx->dMats;
    P.matProps = ctx->dMatProps;
    P.nMats = ctx->nMats;
    P.profiles = ctx->dProfiles;
    P.profileIcdf = ctx->dProfileIcdf;
    P.nProfiles = ctx->nProfiles;
    P.lightPos = ctx->dLightPos;
    P.lightNrm = ctx->dLightNrm;
    P.lightArea = ctx->dLightArea;
    P.lightFlux = ctx->dLightFlux;
    P.alias = ctx->dAlias;
    P.primToLight = ctx->dPrimToLight;
    P.lightEmission = ctx->dLightEmission;
    P.nLights = ctx->nLights;
    P.invWeightsSum = ctx->invWeightsSum;
    P.maxBounces = o.max_bounces;
    P.tileSize = o.tile_size ? o.tile_size : 512;
    P.hwss = o.hwss;
    P.flags = o.flags;
    const bool nee = o.do_nee != 0;
    // light types without an environment map or analytic lights (PLTPT.cpp:230-232)
    P.opt = (o.hwss_do_mis ? plt::kPtHwssMis : 0u) | (o.use_direct_light ? plt::kPtUseDirect : 0u) |
            (o.use_emissive_lights && ctx->nLights ? plt::kPtUseEmissive : 0u) | (nee ? plt::kPtDoNee : 0u) |
            (nee && o.do_mis ? plt::kPtDoMis : 0u) | (o.do_russian_roulette ? plt::kPtDoRR : 0u) |
            (nee && o.nee_use_per_tile_sg ? plt::kPtPerTileSg : 0u) | (o.do_importance_sample_emitters ? plt::kPtImportanceEmit : 0u) |
            (nee && o.do_mnee ? plt::kPtDoMnee : 0u) | (learned ? plt::kPtLearned : 0u);
    P.propNet = ctx->dPropBf16;
    P.matFeat = ctx->dMatFeat;
    P.propProb = o.learned_proposal_prob;
    P.wpss = learned ? static_cast<float*>(ctx->dPtMix) : nullptr;
    // deferred manifold walks: one task slot per path and frame (a fuller queue walks inline)
    if (nee && o.do_mnee) {
        const size_t taskBytes = (size_t)npix * plt::kMneeTaskBytes;
        if (ctx->mneeBytes < taskBytes) {
            cudaFree(ctx->dMneeTasks);
            ctx->dMneeTasks = nullptr;
            ctx->mneeBytes = 0;
            PLT_CUDA(ctx, cudaMalloc(&ctx->dMneeTasks, taskBytes));
            ctx->mneeBytes = taskBytes;
        }
        P.mneeTasks = ctx->dMneeTasks;
        P.mneeCap = npix;
    } else {
        P.mneeTasks = nullptr;
        P.mneeCap = 0;
    }
    P.mneeMaxOccluders = o.mnee_max_occluders;
    P.mneeMaxIterations = o.mnee_max_iterations;
    P.mneeThreshold = o.mnee_solver_threshold;
    P.sourcingArea = o.sourcing_area_from_emissive_geometry;
    P.maxBeamOmega = o.sourcing_max_beam_omega;
    P.cam = *camera;
    P.width = width;
    P.height = height;
    P.npix = npix;
    P.stats = ctx->dPtStats;
    P.status = ctx->dStatus;
    PLT_CUDA(ctx, cudaMemsetAsync(P.accum, 0, sizeof(double) * 3 * (size_t)npix, st));
    for (uint32_t f = 0; f < frame_count; ++f) {
        PLT_CUDA(ctx, cudaMemsetAsync(ctx->dPtStats, 0, 4 * sizeof(unsigned long long), st));
        P.frame = frame_begin + f;
        PLT_CUDA(ctx, plt::launchRenderFrame(P, ctx->numSMs, st));
    }
    PLT_CUDA(ctx, plt::launchResolve(P.accum, npix, frame_count, out_rgba, ctx->numSMs, st));
    return PLT_OK;
}

plt_status plt_render_stats(plt_context* ctx, uint64_t* out4) {
    if (!ctx || !out4) return PLT_INVALID_ARG;
    unsigned long long h[4] = {0, 0, 0, 0};
    if (ctx->dPtStats) PLT_CUDA(ctx, cudaMemcpy(h, ctx->dPtStats, sizeof(h), cudaMemcpyDeviceToHost));
    out4[0] = ctx->ptNpix;
    out4[1] = h[0];
    out4[2] = h[1];
    out4[3] = h[2];
    return PLT_OK;
}

plt_status plt_render_bounces(plt_context* ctx, uint32_t* prim, uint32_t* lobe, uint32_t* flags) {
    if (!ctx || !ctx->dPt) return PLT_INVALID_ARG;
    const size_t n = ctx->ptNpix, nb = (size_t)ctx->ptMaxB + 1;
    std::vector<uint32_t> plane(n * nb);
    const uint32_t* src[3] = {ctx->pt.bPrim, ctx->pt.bLobe, ctx->pt.bFlags};
    uint32_t* dst[3] = {prim, lobe, flags};
    PLT_CUDA(ctx, cudaDeviceSynchronize());
    std::vector<uint8_t> present(n * nb, 0);
    {
        // a record exists for bounce b of a path when bounce b-1 continued the path
        std::vector<uint32_t> fl(n * nb);
        PLT_CUDA(ctx, cudaMemcpy(fl.data(), ctx->pt.bFlags, 4 * n * nb, cudaMemcpyDeviceToHost));
        std::vector<uint32_t> lens(n);
        PLT_CUDA(ctx, cudaMemcpy(lens.data(), ctx->pt.plen, 4 * n, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; ++i) {
            // records 0 .. len hold data (len is the index of the final miss/terminated record)
            const size_t last = std::min<size_t>(lens[i], nb - 1);
            for (size_t b = 0; b <= last; ++b) present[i * nb + b] = 1;
        }
    }
    for (int k = 0; k < 3; ++k) {
        if (!dst[k]) continue;
        PLT_CUDA(ctx, cudaMemcpy(plane.data(), src[k], 4 * n * nb, cudaMemcpyDeviceToHost));
        for (size_t i = 0; i < n; ++i)
            for (size_t b = 0; b < nb; ++b)
                dst[k][i * nb + b] = present[i * nb + b] ? plane[b * n + i] : (k == 0 ? 0xFFFFFFFFu : 0u);
    }
    return PLT_OK;
}

}  // extern "C"
