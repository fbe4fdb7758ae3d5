// The context's scene set: host-side scene construction (BVH, leaf-ordered triangles, shading
// attributes), the per-scene emissive-triangle light collections with the power sampler's alias
// tables, and the upload of all scenes as one combined set of device arrays (node, triangle, vertex
// and light indices rebased; each scene keeps its root, triangle range and light range).  Paths
// cited are inside ssteinberg/PLTFalcor.
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


// Emissive triangles of one scene (materials with an emission profile, in primitive order), their
// face normal and area (computeFaceNormalAndAreaW, Scene/Scene.slang:482-497) and luminous flux
// luminance(profile rgb) * area * pi (Scene/Lights/FinalizeIntegration.cs.slang:60-110), with the
// scene's alias table (scene-local light indices).
struct SceneLights {
    std::vector<float> pos, nrm, area, flux;
    std::vector<uint32_t> emission, tri;
    std::vector<uint2> table;
    float invWeightsSum = 0.f;
};
plt_status collectLights(const plt_context* ctx, const plt_scene_host& sc, SceneLights& L) {
    for (uint32_t t = 0; t < sc.nTris; ++t) {
        const uint32_t m = sc.triMat[t];
        if (m >= ctx->hMats.size()) return PLT_BAD_MATERIAL;
        const plt_material_record& r = ctx->hMats[m];
        if (r.type != PLT_MATERIAL_DIFFUSE || r.emission_spectral_id == PLT_NO_SPECTRAL_PROFILE) continue;
        L.tri.push_back(t);
    }
    const uint32_t nl = (uint32_t)L.tri.size();
    L.pos.resize(9 * (size_t)nl);
    L.nrm.resize(3 * (size_t)nl);
    L.area.resize(nl);
    L.flux.resize(nl);
    L.emission.resize(nl);
    for (uint32_t l = 0; l < nl; ++l) {
        const uint32_t t = L.tri[l];
        V3 p[3];
        for (int k = 0; k < 3; ++k) {
            const float* v = &sc.pos[3 * (size_t)sc.idx[3 * (size_t)t + k]];
            p[k] = {v[0], v[1], v[2]};
            std::memcpy(&L.pos[9 * (size_t)l + 3 * k], v, 12);
        }
        const V3 N = crossv(sub(p[1], p[0]), sub(p[2], p[0]));
        const float len = lengthv(N);
        const V3 n = storedNormal({N.x / len, N.y / len, N.z / len});
        L.nrm[3 * (size_t)l] = n.x;
        L.nrm[3 * (size_t)l + 1] = n.y;
        L.nrm[3 * (size_t)l + 2] = n.z;
        L.area[l] = 0.5f * len;
        const uint32_t em = ctx->hMats[sc.triMat[t]].emission_spectral_id;
        L.emission[l] = em;
        float rgb[3] = {0.f, 0.f, 0.f};
        if (em < ctx->hProfiles.size())
            for (int c = 0; c < 3; ++c) rgb[c] = std::max(0.f, ctx->hProfiles[em].rgb[c]);
        const float lum = rgb[0] * 0.2126f + rgb[1] * 0.7152f + rgb[2] * 0.0722f;
        L.flux[l] = lum * L.area[l] * 3.14159265358979323846f;
    }
    buildAliasTable(L.flux, L.table, L.invWeightsSum);
    return PLT_OK;
}

// Geometry of one scene: validation, the SAH BVH and the triangles in leaf order.
plt_status buildSceneHost(const float* vertices, uint32_t nVerts, const uint32_t* indices, uint32_t nTris, const uint32_t* material,
                          plt_scene_host& sc) {
    if (nTris > 0 && (!vertices || !indices)) return PLT_INVALID_ARG;
    if (nTris >= (1u << 27)) return PLT_NOT_SUPPORTED;  // leaf encoding holds 27-bit triangle offsets
    std::vector<float> tv((size_t)nTris * 9);
    for (uint32_t t = 0; t < nTris; ++t)
        for (int k = 0; k < 3; ++k) {
            const uint32_t vi = indices[3 * (size_t)t + k];
            if (vi >= nVerts) return PLT_INVALID_ARG;
            for (int a = 0; a < 3; ++a) {
                const float x = vertices[3 * (size_t)vi + a];
                if (!std::isfinite(x)) return PLT_NAN_INPUT;
                tv[9 * (size_t)t + 3 * k + a] = x;
            }
        }
    std::vector<uint32_t> order;
    plt::buildBvh(tv.data(), nTris, sc.nodes, order, &sc.stats);
    sc.tris.resize((size_t)nTris * 3);
    for (uint32_t s = 0; s < nTris; ++s) {
        const uint32_t t = order[s];
        const float* p = &tv[9 * (size_t)t];
        float idBits;
        std::memcpy(&idBits, &t, 4);
        sc.tris[3 * s] = make_float4(p[0], p[1], p[2], idBits);
        sc.tris[3 * s + 1] = make_float4(p[3], p[4], p[5], 0.f);
        sc.tris[3 * s + 2] = make_float4(p[6], p[7], p[8], 0.f);
    }
    sc.nVerts = nVerts;
    sc.nTris = nTris;
    sc.pos.assign(vertices, vertices + 3 * (size_t)nVerts);
    sc.idx.assign(indices, indices + 3 * (size_t)nTris);
    sc.triMat.assign(nTris, 0u);
    if (material && nTris) std::memcpy(sc.triMat.data(), material, sizeof(uint32_t) * nTris);
    sc.shaded = false;
    return PLT_OK;
}

plt_status setSceneShading(plt_scene_host& sc, const float* normals, const float* tangents, uint32_t nVerts, const uint32_t* triInst) {
    if (!normals || nVerts != sc.nVerts || sc.nTris == 0) return PLT_INVALID_ARG;
    for (size_t i = 0; i < 3 * (size_t)nVerts; ++i)
        if (!std::isfinite(normals[i])) return PLT_NAN_INPUT;
    sc.nrm.assign(normals, normals + 3 * (size_t)nVerts);
    if (tangents) sc.tan.assign(tangents, tangents + 4 * (size_t)nVerts);
    else sc.tan.clear();
    sc.triInst.assign(sc.nTris, 0u);
    if (triInst) std::memcpy(sc.triInst.data(), triInst, sizeof(uint32_t) * sc.nTris);
    sc.shaded = true;
    return PLT_OK;
}

// EnvMap::setRotation (Scene/Lights/EnvMap.cpp:60-71): rotation degrees (x, y, z) to
// toWorld = Rx(x) Ry(y) Rz(z) (row-major); toLocal is its transpose.
void envRotation(const float deg[3], float toWorld[9], float toLocal[9]) {
    const float k = 3.14159265358979323846f / 180.f;
    const float a = deg[0] * k, b = deg[1] * k, c = deg[2] * k;
    const float ca = std::cos(a), sa = std::sin(a), cb = std::cos(b), sb = std::sin(b), cc = std::cos(c), sc = std::sin(c);
    const float M[9] = {cb * cc, -cb * sc, sb,
                        ca * sc + sa * sb * cc, ca * cc - sa * sb * sc, -sa * cb,
                        sa * sc - ca * sb * cc, sa * cc + ca * sb * sc, ca * cb};
    for (int r = 0; r < 3; ++r)
        for (int q = 0; q < 3; ++q) {
            toWorld[3 * r + q] = M[3 * r + q];
            toLocal[3 * r + q] = M[3 * q + r];
        }
}

}  // namespace

void pltReleaseEnv(plt_context* ctx) {
    cudaFree(ctx->dALights);
    ctx->dALights = nullptr;
    ctx->nALights = 0;
    cudaFree(ctx->dEnvTex);
    cudaFree(ctx->dEnvImp);
    ctx->dEnvTex = nullptr;
    ctx->dEnvImp = nullptr;
    ctx->envTexCap = 0;
    ctx->env = plt::EnvDev{};
    ctx->hasEnv = false;
}

// Uploads the scene set as one set of device arrays.  Geometry: BVH nodes with child indices
// rebased by the scene's first node and leaf triangle offsets by its first triangle, triangles with
// global ids (first triangle + local id), vertex indices rebased by the scene's first vertex.
// Shading (when every scene has it): normals, tangents (zero, i.e. absent, for scenes without),
// geometry instances made unique across scenes, and the light collections concatenated with
// global primitive-to-light indices.
plt_status pltUploadScenes(plt_context* ctx) {
    plt_status st;
    const size_t ns = ctx->scenes.size();
    if (ctx->geometryDirty) {
        std::vector<plt::BvhNode> nodes;
        std::vector<float4> tris;
        std::vector<uint32_t> triMat, idx;
        std::vector<float> pos;
        ctx->slots.assign(ns, plt_scene_slot{});
        for (size_t i = 0; i < ns; ++i) {
            const plt_scene_host& sc = ctx->scenes[i];
            const uint32_t nodeBase = (uint32_t)nodes.size(), triBase = (uint32_t)(tris.size() / 3), vertBase = (uint32_t)(pos.size() / 3);
            if ((uint64_t)triBase + sc.nTris >= (1u << 27)) return PLT_NOT_SUPPORTED;
            auto rebase = [&](int32_t c) -> int32_t {
                if (c == plt::kNoChild) return c;
                if (c >= 0) return c + (int32_t)nodeBase;
                const uint32_t v = (uint32_t)~c;
                return ~(int32_t)((((v >> 4) + triBase) << 4) | (v & 15u));
            };
            for (plt::BvhNode n : sc.nodes) {
                n.left = rebase(n.left);
                n.right = rebase(n.right);
                nodes.push_back(n);
            }
            for (size_t k = 0; k < sc.tris.size(); ++k) {
                float4 v = sc.tris[k];
                if (k % 3 == 0) {
                    uint32_t id;
                    std::memcpy(&id, &v.w, 4);
                    id += triBase;
                    std::memcpy(&v.w, &id, 4);
                }
                tris.push_back(v);
            }
            triMat.insert(triMat.end(), sc.triMat.begin(), sc.triMat.end());
            for (uint32_t v : sc.idx) idx.push_back(v + vertBase);
            pos.insert(pos.end(), sc.pos.begin(), sc.pos.end());
            ctx->slots[i].root = nodeBase;
            ctx->slots[i].triBase = triBase;
        }
        cudaFree(ctx->dNodes);
        cudaFree(ctx->dTris);
        cudaFree(ctx->dTriMaterial);
        ctx->dNodes = nullptr;
        ctx->dTris = nullptr;
        ctx->dTriMaterial = nullptr;
        ctx->nTris = 0;
        if (!nodes.empty()) {
            PLT_CUDA(ctx, cudaMalloc(&ctx->dNodes, sizeof(plt::BvhNode) * nodes.size()));
            PLT_CUDA(ctx, cudaMemcpy(ctx->dNodes, nodes.data(), sizeof(plt::BvhNode) * nodes.size(), cudaMemcpyHostToDevice));
        }
        if ((st = upload(ctx, ctx->dTris, tris.data(), tris.size())) != PLT_OK) return st;
        if ((st = upload(ctx, ctx->dTriMaterial, triMat.data(), triMat.size())) != PLT_OK) return st;
        if ((st = upload(ctx, ctx->dPos, pos.data(), pos.size())) != PLT_OK) return st;
        if ((st = upload(ctx, ctx->dIdx, idx.data(), idx.size())) != PLT_OK) return st;
        ctx->nTris = (uint32_t)triMat.size();
        ctx->nVerts = ns ? ctx->scenes.back().nVerts : 0;
        ctx->bvhStats = ns ? ctx->scenes.back().stats : plt::BvhBuildStats{};
        ctx->geometryDirty = false;
        ctx->shadingDirty = true;
    }
    if (ctx->shadingDirty) {
        ctx->shadingReady = false;
        bool all = ns > 0 && ctx->nTris > 0, anyTan = false;
        for (const plt_scene_host& sc : ctx->scenes) {
            all = all && sc.shaded;
            anyTan = anyTan || !sc.tan.empty();
        }
        if (all) {
            std::vector<float> nrm, tan, lpos, lnrm, larea, lflux;
            std::vector<uint32_t> inst, p2l(ctx->nTris, 0xFFFFFFFFu), lem, lactive;
            std::vector<uint2> alias;
            uint32_t instBase = 0;
            for (size_t i = 0; i < ns; ++i) {
                const plt_scene_host& sc = ctx->scenes[i];
                nrm.insert(nrm.end(), sc.nrm.begin(), sc.nrm.end());
                if (anyTan) {
                    if (sc.tan.empty()) tan.insert(tan.end(), 4 * (size_t)sc.nVerts, 0.f);
                    else tan.insert(tan.end(), sc.tan.begin(), sc.tan.end());
                }
                uint32_t maxInst = 0;
                for (uint32_t g : sc.triInst) {
                    inst.push_back(g + instBase);
                    maxInst = std::max(maxInst, g);
                }
                instBase += maxInst + 1;
                SceneLights L;
                if ((st = collectLights(ctx, sc, L)) != PLT_OK) return st;
                const uint32_t lightBase = (uint32_t)larea.size(), nl = (uint32_t)L.area.size();
                for (uint32_t l = 0; l < nl; ++l) p2l[ctx->slots[i].triBase + L.tri[l]] = lightBase + l;
                lpos.insert(lpos.end(), L.pos.begin(), L.pos.end());
                lnrm.insert(lnrm.end(), L.nrm.begin(), L.nrm.end());
                larea.insert(larea.end(), L.area.begin(), L.area.end());
                lflux.insert(lflux.end(), L.flux.begin(), L.flux.end());
                lem.insert(lem.end(), L.emission.begin(), L.emission.end());
                alias.insert(alias.end(), L.table.begin(), L.table.end());
                // LightCollection's active triangle list (flux > 0, LightCollection.cpp:512-524)
                ctx->slots[i].activeBase = (uint32_t)lactive.size();
                for (uint32_t l = 0; l < nl; ++l)
                    if (L.flux[l] > 0.f) lactive.push_back(lightBase + l);
                ctx->slots[i].nActive = (uint32_t)lactive.size() - ctx->slots[i].activeBase;
                ctx->slots[i].lightBase = lightBase;
                ctx->slots[i].nLights = nl;
                ctx->slots[i].invWeightsSum = L.invWeightsSum;
            }
            if ((st = upload(ctx, ctx->dNrm, nrm.data(), nrm.size())) != PLT_OK) return st;
            if ((st = upload(ctx, ctx->dTan, tan.data(), tan.size())) != PLT_OK) return st;
            if ((st = upload(ctx, ctx->dTriInst, inst.data(), inst.size())) != PLT_OK) return st;
            if ((st = upload(ctx, ctx->dLightPos, lpos.data(), lpos.size())) != PLT_OK) return st;
            if ((st = upload(ctx, ctx->dLightNrm, lnrm.data(), lnrm.size())) != PLT_OK) return st;
            if ((st = upload(ctx, ctx->dLightArea, larea.data(), larea.size())) != PLT_OK) return st;
            if ((st = upload(ctx, ctx->dLightFlux, lflux.data(), lflux.size())) != PLT_OK) return st;
            if ((st = upload(ctx, ctx->dAlias, alias.data(), alias.size())) != PLT_OK) return st;
            if ((st = upload(ctx, ctx->dLightEmission, lem.data(), lem.size())) != PLT_OK) return st;
            if ((st = upload(ctx, ctx->dPrimToLight, p2l.data(), p2l.size())) != PLT_OK) return st;
            if ((st = upload(ctx, ctx->dLightActive, lactive.data(), lactive.size())) != PLT_OK) return st;
            ctx->nLights = (uint32_t)larea.size();
            ctx->invWeightsSum = ctx->slots[0].invWeightsSum;
            ctx->shadingReady = true;
        }
        ctx->shadingDirty = false;
    }
    return PLT_OK;
}

extern "C" {

plt_status plt_set_scene(plt_context* ctx, const float* vertices, uint32_t nVerts, const uint32_t* indices, uint32_t nTris,
                         const uint32_t* material) {
    if (!ctx) return PLT_INVALID_ARG;
    plt_scene_host sc;
    const plt_status s = buildSceneHost(vertices, nVerts, indices, nTris, material, sc);
    if (s != PLT_OK) return s;
    ctx->scenes.clear();
    ctx->scenes.push_back(std::move(sc));
    ctx->geometryDirty = true;
    return pltUploadScenes(ctx);
}

plt_status plt_set_scene_shading(plt_context* ctx, const float* normals, const float* tangents, uint32_t n_vertices,
                                 const uint32_t* tri_instance) {
    if (!ctx || ctx->scenes.empty()) return PLT_INVALID_ARG;
    const plt_status s = setSceneShading(ctx->scenes.back(), normals, tangents, n_vertices, tri_instance);
    if (s != PLT_OK) return s;
    ctx->shadingDirty = true;
    return pltUploadScenes(ctx);
}

plt_status plt_add_scene(plt_context* ctx, const plt_scene_desc* desc, uint32_t* out_scene) {
    if (!ctx || !desc || desc->n_triangles == 0) return PLT_INVALID_ARG;
    if (ctx->scenes.size() >= PLT_MAX_SCENES) return PLT_NOT_SUPPORTED;
    plt_scene_host sc;
    plt_status s = buildSceneHost(desc->positions, desc->n_vertices, desc->indices, desc->n_triangles, desc->tri_material, sc);
    if (s != PLT_OK) return s;
    if ((s = setSceneShading(sc, desc->normals, desc->tangents, desc->n_vertices, desc->tri_instance)) != PLT_OK) return s;
    if (out_scene) *out_scene = (uint32_t)ctx->scenes.size();
    ctx->scenes.push_back(std::move(sc));
    ctx->geometryDirty = true;
    return PLT_OK;
}

plt_status plt_clear_scenes(plt_context* ctx) {
    if (!ctx) return PLT_INVALID_ARG;
    ctx->scenes.clear();
    ctx->geometryDirty = true;
    return pltUploadScenes(ctx);
}

// Scene::setEnvMap + EnvMap (Scene/Lights/EnvMap.cpp) + EnvMapSampler::createImportanceMap
// (Rendering/Lights/EnvMapSampler.cpp:85-120): uploads the lat-long map and builds the sampler's
// 512 x 512 importance map (64 subsamples per texel) and its mips on the device.
plt_status plt_set_env_map(plt_context* ctx, const float* pixels, uint32_t width, uint32_t height, uint32_t channels,
                           float intensity, const float* tint, const float* rotation_deg) {
    if (!ctx || !pixels || width == 0 || height == 0 || width > 16384 || height > 16384) return PLT_INVALID_ARG;
    if (channels != 3 && channels != 4) return PLT_INVALID_ARG;
    if (!std::isfinite(intensity) || intensity < 0.f) return PLT_INVALID_ARG;
    const float one[3] = {1.f, 1.f, 1.f}, zero[3] = {0.f, 0.f, 0.f};
    const float* tn = tint ? tint : one;
    const float* rot = rotation_deg ? rotation_deg : zero;
    for (int i = 0; i < 3; ++i)
        if (!std::isfinite(tn[i]) || tn[i] < 0.f || !std::isfinite(rot[i])) return PLT_INVALID_ARG;
    const size_t n = (size_t)width * height;
    std::vector<float4> tex(n);
    for (size_t i = 0; i < n; ++i) {
        const float* q = pixels + channels * i;
        if (!(std::isfinite(q[0]) && std::isfinite(q[1]) && std::isfinite(q[2])) || q[0] < 0.f || q[1] < 0.f || q[2] < 0.f)
            return PLT_INVALID_ARG;
        tex[i] = make_float4(q[0], q[1], q[2], channels == 4 ? q[3] : 1.f);
    }
    if (ctx->envTexCap < n) {
        cudaFree(ctx->dEnvTex);
        ctx->dEnvTex = nullptr;
        ctx->envTexCap = 0;
        PLT_CUDA(ctx, cudaMalloc(&ctx->dEnvTex, sizeof(float4) * n));
        ctx->envTexCap = n;
    }
    PLT_CUDA(ctx, cudaMemcpy(ctx->dEnvTex, tex.data(), sizeof(float4) * n, cudaMemcpyHostToDevice));
    plt::EnvDev E{};
    E.impDim = plt::kEnvImportanceDim;
    uint32_t off = 0, mip = 0;
    for (uint32_t d = E.impDim; d >= 1; d >>= 1, ++mip) {
        E.mipOff[mip] = off;
        off += d * d;
        E.impBaseMip = mip;
    }
    if (!ctx->dEnvImp) PLT_CUDA(ctx, cudaMalloc(&ctx->dEnvImp, sizeof(float) * off));
    E.tex = ctx->dEnvTex;
    E.width = width;
    E.height = height;
    E.imp = ctx->dEnvImp;
    envRotation(rot, E.toWorld, E.toLocal);
    for (int i = 0; i < 3; ++i) E.scale[i] = intensity * tn[i];
    PLT_CUDA(ctx, plt::launchEnvImportance(E, 0));
    PLT_CUDA(ctx, cudaStreamSynchronize(0));
    ctx->env = E;
    ctx->hasEnv = true;
    return PLT_OK;
}

plt_status plt_clear_env_map(plt_context* ctx) {
    if (!ctx) return PLT_INVALID_ARG;
    cudaFree(ctx->dEnvTex);
    cudaFree(ctx->dEnvImp);
    ctx->dEnvTex = nullptr;
    ctx->dEnvImp = nullptr;
    ctx->envTexCap = 0;
    ctx->env = plt::EnvDev{};
    ctx->hasEnv = false;
    return PLT_OK;
}

// The scene's analytic lights (LightData, Scene/Lights/Light.cpp): validated and uploaded with the
// inverse-transpose of each transform (AnalyticAreaLight::update, Light.cpp:341-346) and the area
// lights' world normal (LightHelpers.slang:112, 164).
plt_status plt_set_analytic_lights(plt_context* ctx, const plt_analytic_light* lights, uint32_t count) {
    if (!ctx || (count > 0 && !lights)) return PLT_INVALID_ARG;
    std::vector<plt::AnalyticLightDev> h(count);
    for (uint32_t i = 0; i < count; ++i) {
        const plt_analytic_light& l = lights[i];
        if (l.type > PLT_LIGHT_SPHERE) return PLT_INVALID_ARG;
        if (l.intensity_spectral_id != PLT_NO_SPECTRAL_PROFILE && l.intensity_spectral_id >= ctx->nProfiles) return PLT_INVALID_ARG;
        plt::AnalyticLightDev& d = h[i];
        std::memset(&d, 0, sizeof(d));
        for (int k = 0; k < 3; ++k) { d.pos[k] = l.pos[k]; d.dir[k] = l.dir[k]; }
        d.type = l.type;
        d.spectrumId = l.intensity_spectral_id;
        d.openingAngle = l.opening_angle;
        d.cosOpeningAngle = l.cos_opening_angle;
        d.penumbraAngle = l.penumbra_angle;
        d.cosSubtendedAngle = l.cos_subtended_angle;
        d.surfaceArea = l.surface_area;
        for (int k = 0; k < 12; ++k) d.xf[k] = l.transform[k];
        // inverse-transpose of the 3x3 part (cofactor matrix / determinant)
        const double a[9] = {l.transform[0], l.transform[1], l.transform[2], l.transform[4], l.transform[5], l.transform[6],
                             l.transform[8], l.transform[9], l.transform[10]};
        const double cof[9] = {a[4] * a[8] - a[5] * a[7], a[5] * a[6] - a[3] * a[8], a[3] * a[7] - a[4] * a[6],
                               a[2] * a[7] - a[1] * a[8], a[0] * a[8] - a[2] * a[6], a[1] * a[6] - a[0] * a[7],
                               a[1] * a[5] - a[2] * a[4], a[2] * a[3] - a[0] * a[5], a[0] * a[4] - a[1] * a[3]};
        const double det = a[0] * cof[0] + a[1] * cof[1] + a[2] * cof[2];
        if (l.type >= PLT_LIGHT_DISTANT && !(std::fabs(det) > 0.0)) return PLT_INVALID_ARG;
        for (int k = 0; k < 9; ++k) d.xfIT[k] = std::fabs(det) > 0.0 ? (float)(cof[k] / det) : 0.f;
        const float n[3] = {d.xfIT[2], d.xfIT[5], d.xfIT[8]};
        const float len = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        for (int k = 0; k < 3; ++k) d.nrm[k] = len > 0.f ? n[k] / len : 0.f;
    }
    cudaFree(ctx->dALights);
    ctx->dALights = nullptr;
    ctx->nALights = 0;
    if (count) {
        PLT_CUDA(ctx, cudaMalloc(&ctx->dALights, sizeof(plt::AnalyticLightDev) * count));
        PLT_CUDA(ctx, cudaMemcpy(ctx->dALights, h.data(), sizeof(plt::AnalyticLightDev) * count, cudaMemcpyHostToDevice));
    }
    ctx->nALights = count;
    return PLT_OK;
}

plt_status plt_env_map_query(plt_context* ctx, const float* u, const float* dirs, uint32_t n, float* out, void* stream) {
    if (!ctx || (n > 0 && (!u || !out))) return PLT_INVALID_ARG;
    if (!ctx->hasEnv) return PLT_INVALID_ARG;
    PLT_CUDA(ctx, plt::launchEnvQuery(ctx->env, u, dirs, n, out, static_cast<cudaStream_t>(stream)));
    return PLT_OK;
}

}  // extern "C"
