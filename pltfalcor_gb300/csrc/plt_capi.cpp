// C ABI of libplt_gb300.so (declared in include/plt_gb300.h): context, material and spectral
// tables, batched BSDF launches, status.  No exception crosses the ABI.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "plt_bvh.h"
#include "plt_host.h"
#include "plt_internal.h"

#include "plt_context.h"
#include "plt_nvtx.h"

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

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

}  // namespace

extern "C" {

uint32_t plt_abi_version(void) { return PLT_ABI_VERSION; }

const char* plt_status_string(plt_status s) {
    switch (s) {
    case PLT_OK: return "ok";
    case PLT_INVALID_ARG: return "invalid argument";
    case PLT_OOM: return "out of device memory";
    case PLT_QUEUE_TIMEOUT: return "queue wait timed out";
    case PLT_NAN_INPUT: return "non-finite input";
    case PLT_CUDA_ERROR: return "CUDA error";
    case PLT_NOT_SUPPORTED: return "not supported";
    case PLT_BAD_MATERIAL: return "bad material";
    case PLT_TOO_LARGE: return "batch larger than the allocation-free scratch capacity";
    case PLT_BOUNDS_VIOLATION: return "index outside its buffer (bounds-check build)";
    }
    return "unknown status";
}

plt_status plt_options_default(plt_options* o) {
    if (!o) return PLT_INVALID_ARG;
    std::memset(o, 0, sizeof(*o));
    o->max_bounces = 32;
    o->tile_size = 512;
    o->hwss = 4;
    o->hwss_do_mis = 1;
    o->sourcing_area_from_emissive_geometry = 1.f;
    o->sourcing_max_beam_omega = .025f;
    o->use_direct_light = 1;
    o->use_env_light = 1;
    o->use_emissive_lights = 1;
    o->use_analytic_lights = 1;
    o->do_nee = 1;
    o->do_mis = 1;
    o->do_russian_roulette = 1;
    o->nee_use_per_tile_sg = 0;
    o->do_importance_sample_emitters = 1;
    o->do_mnee = 1;
    o->mnee_max_occluders = 2;
    o->mnee_max_iterations = 60;
    o->mnee_solver_threshold = 5e-5f;
    o->flags = 0;
    o->learned_proposal = 0;
    o->learned_proposal_prob = .5f;
    o->emissive_sampler = 2u;
    o->debug_view = PLT_DEBUG_VIEW_NONE;
    o->debug_view_intensity = 1.f;
    o->alpha_masking = 1;
    o->sample_generator = PLT_SAMPLE_GENERATOR_UNIFORM;
    return PLT_OK;
}

plt_status plt_create(const plt_options* options, plt_context** out) {
    if (!out) return PLT_INVALID_ARG;
    *out = nullptr;
    plt_context* ctx = new (std::nothrow) plt_context();
    if (!ctx) return PLT_OOM;
    if (options) ctx->opt = *options;
    else plt_options_default(&ctx->opt);
    if (ctx->opt.hwss < 1 || ctx->opt.hwss > PLT_MAX_HWSS) { delete ctx; return PLT_INVALID_ARG; }
    // debugView (DebugViewType), sampleGenerator (SampleGeneratorType) value ranges
    if (ctx->opt.debug_view > PLT_DEBUG_VIEW_MNEE_BOUNCES || ctx->opt.sample_generator > PLT_SAMPLE_GENERATOR_UNIFORM) {
        delete ctx;
        return PLT_INVALID_ARG;
    }
    // the albedo and roughness views need BSDFProperties.albedo / .roughness, which are not built
    if (ctx->opt.debug_view == PLT_DEBUG_VIEW_ALBEDO || ctx->opt.debug_view == PLT_DEBUG_VIEW_ROUGHNESS) {
        delete ctx;
        return PLT_NOT_SUPPORTED;
    }
    // PLTPT offers the Uniform and Power emissive samplers (PLTPT.cpp:80-83, 401-409)
    if (ctx->opt.emissive_sampler != 0u && ctx->opt.emissive_sampler != 2u) {
        const bool bvh = ctx->opt.emissive_sampler == 1u;
        delete ctx;
        return bvh ? PLT_NOT_SUPPORTED : PLT_INVALID_ARG;
    }
    cudaError_t e = cudaGetDevice(&ctx->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&ctx->numSMs, cudaDevAttrMultiProcessorCount, ctx->device);
    if (e == cudaSuccess) e = cudaMalloc(&ctx->dStatus, sizeof(uint32_t) * plt::kStatusWords);
    if (e == cudaSuccess) e = cudaMemset(ctx->dStatus, 0, sizeof(uint32_t) * plt::kStatusWords);
    if (e != cudaSuccess) {
        const plt_status s = e == cudaErrorMemoryAllocation ? PLT_OOM : PLT_CUDA_ERROR;
        if (ctx->dStatus) cudaFree(ctx->dStatus);
        delete ctx;
        return s;
    }
    *out = ctx;
    return PLT_OK;
}

plt_status plt_destroy(plt_context* ctx) {
    if (!ctx) return PLT_INVALID_ARG;
    // the host pipeline's streams may still run kernels that read the buffers below: drain them first
    pltReleaseHostPipeline(ctx);
    cudaFree(ctx->dMats);
    cudaFree(ctx->dMatType);
    cudaFree(ctx->dProfiles);
    cudaFree(ctx->dStatus);
    cudaFree(ctx->dScratch);
    cudaFree(ctx->dNodes);
    cudaFree(ctx->dTris);
    cudaFree(ctx->dTriMaterial);
    pltReleaseRenderState(ctx);
    pltReleaseProposal(ctx);
    pltReleaseEnv(ctx);
    delete ctx;
    return PLT_OK;
}

int plt_last_cuda_error(const plt_context* ctx) { return ctx ? ctx->lastCudaError : 0; }

plt_status plt_set_spectral_profiles(plt_context* ctx, const plt_spectral_profile* profiles, uint32_t count) {
    if (!ctx || (count > 0 && !profiles)) return PLT_INVALID_ARG;
    if (count > 64) return PLT_NOT_SUPPORTED;  // staged whole into shared memory by each CTA
    std::vector<pltdev::DevProfile> h(count);
    for (uint32_t i = 0; i < count; ++i) {
        const plt_spectral_profile& s = profiles[i];
        if (s.bins > PLT_SPECTRAL_MAX_BINS) return PLT_INVALID_ARG;
        std::memset(&h[i], 0, sizeof(h[i]));
        h[i].intensity = s.intensity;
        h[i].minl = s.min_wavelength;
        h[i].maxl = s.max_wavelength;
        h[i].bins = s.bins;
        std::memcpy(h[i].pdf, s.pdf, sizeof(h[i].pdf));
    }
    if (count > ctx->capProfiles) {
        cudaFree(ctx->dProfiles);
        ctx->dProfiles = nullptr;
        ctx->capProfiles = 0;
        PLT_CUDA(ctx, cudaMalloc(&ctx->dProfiles, sizeof(pltdev::DevProfile) * count));
        ctx->capProfiles = count;
    }
    if (count) PLT_CUDA(ctx, cudaMemcpy(ctx->dProfiles, h.data(), sizeof(pltdev::DevProfile) * count, cudaMemcpyHostToDevice));
    // inverse CDFs for emission importance sampling (Scene.sampleSpectrum)
    cudaFree(ctx->dProfileIcdf);
    ctx->dProfileIcdf = nullptr;
    if (count) {
        std::vector<float> icdf((size_t)count * PLT_SPECTRAL_MAX_BINS);
        for (uint32_t i = 0; i < count; ++i) std::memcpy(&icdf[(size_t)i * PLT_SPECTRAL_MAX_BINS], profiles[i].icdf, sizeof(profiles[i].icdf));
        PLT_CUDA(ctx, cudaMalloc(&ctx->dProfileIcdf, sizeof(float) * icdf.size()));
        PLT_CUDA(ctx, cudaMemcpy(ctx->dProfileIcdf, icdf.data(), sizeof(float) * icdf.size(), cudaMemcpyHostToDevice));
    }
    ctx->hProfiles.assign(profiles, profiles + count);
    ctx->nProfiles = count;
    ctx->shadingDirty = true;   // lights depend on materials and profiles
    return PLT_OK;
}

namespace {
// The high bits of a material's type byte for the batch sort: bit 7 set and the work class in bits
// 4..6 when the trip count of its evaluation loop varies between materials of the type, so the
// classify pass gives a warp materials of similar cost (stack layers in fours for multilayers, which
// expose one lobe); 0 for the rest, which are sorted by the query's lobe.
uint32_t batchWorkClass(uint32_t type, const pltdev::DevMaterial& d) {
    if (type != PLT_MATERIAL_MULTILAYERED_STACK) return 0u;
    return 0x80u | (std::min((d.aux > 0u ? d.aux - 1u : 0u) >> 2, 7u) << 4);
}
}  // namespace

plt_status plt_set_materials(plt_context* ctx, const plt_material_record* mats, uint32_t count) {
    if (!ctx || (count > 0 && !mats)) return PLT_INVALID_ARG;
    std::vector<pltdev::DevMaterial> h(count);
    std::vector<uint8_t> types(count);
    for (uint32_t i = 0; i < count; ++i) {
        const plt_status s = plt::decodeMaterial(mats[i], ctx->nProfiles, h[i]);
        if (s != PLT_OK) return s;
        types[i] = (uint8_t)(mats[i].type | batchWorkClass(mats[i].type, h[i]));
    }
    if (count > ctx->capMats) {
        cudaFree(ctx->dMats);
        cudaFree(ctx->dMatType);
        ctx->dMats = nullptr;
        ctx->dMatType = nullptr;
        ctx->capMats = 0;
        PLT_CUDA(ctx, cudaMalloc(&ctx->dMats, sizeof(pltdev::DevMaterial) * count));
        PLT_CUDA(ctx, cudaMalloc(&ctx->dMatType, count));
        ctx->capMats = count;
    }
    if (count) {
        PLT_CUDA(ctx, cudaMemcpy(ctx->dMats, h.data(), sizeof(pltdev::DevMaterial) * count, cudaMemcpyHostToDevice));
        PLT_CUDA(ctx, cudaMemcpy(ctx->dMatType, types.data(), count, cudaMemcpyHostToDevice));
    }
    // per-material property words of the render pass
    cudaFree(ctx->dMatProps);
    ctx->dMatProps = nullptr;
    if (count) {
        std::vector<uint2> props(count);
        for (uint32_t i = 0; i < count; ++i) props[i] = pltMaterialProps(mats[i], h[i]);
        PLT_CUDA(ctx, cudaMalloc(&ctx->dMatProps, sizeof(uint2) * count));
        PLT_CUDA(ctx, cudaMemcpy(ctx->dMatProps, props.data(), sizeof(uint2) * count, cudaMemcpyHostToDevice));
    }
    // learned-proposal features and the list of materials it serves
    cudaFree(ctx->dMatFeat);
    cudaFree(ctx->dPropEnabled);
    ctx->dMatFeat = nullptr;
    ctx->dPropEnabled = nullptr;
    ctx->nPropEnabled = 0;
    if (count) {
        std::vector<float4> feat(count);
        std::vector<uint32_t> enabled;
        for (uint32_t i = 0; i < count; ++i) {
            feat[i] = pltProposalFeatures(mats[i], h[i]);
            if (feat[i].w != 0.f) enabled.push_back(i);
        }
        PLT_CUDA(ctx, cudaMalloc(&ctx->dMatFeat, sizeof(float4) * count));
        PLT_CUDA(ctx, cudaMemcpy(ctx->dMatFeat, feat.data(), sizeof(float4) * count, cudaMemcpyHostToDevice));
        if (!enabled.empty()) {
            PLT_CUDA(ctx, cudaMalloc(&ctx->dPropEnabled, sizeof(uint32_t) * enabled.size()));
            PLT_CUDA(ctx, cudaMemcpy(ctx->dPropEnabled, enabled.data(), sizeof(uint32_t) * enabled.size(), cudaMemcpyHostToDevice));
        }
        ctx->nPropEnabled = (uint32_t)enabled.size();
    }
    ctx->hMats.assign(mats, mats + count);
    ctx->hDevMats = h;
    ctx->nMats = count;
    ctx->shadingDirty = true;   // lights depend on materials and profiles
    return PLT_OK;
}

plt_status plt_spectral_profile_from_samples(const float* wl, const float* values, uint32_t count, float scale, int compute_icdf,
                                             plt_spectral_profile* out) {
    return plt::spectralProfileFromSamples(wl, values, count, scale, compute_icdf, out);
}

plt_status plt_bsdf_batch(plt_context* ctx, const plt_bsdf_queries* q, const plt_bsdf_results* r, uint32_t ops, void* stream) {
    const plt::NvtxRange range("bsdf_batch");
    plt::BatchParams p{};
    int numSMs = 0;
    const plt_status s = plt::fillBatchParams(ctx, q, r, ops, &p, &numSMs);
    if (s != PLT_OK || q->n == 0) return s;
    const size_t need = plt::bsdfScratchBytes(q->n);
    if (need > ctx->scratchCap) {
        // grows once to the largest batch seen; cudaFree waits for every batch still using the old one
        cudaFree(ctx->dScratch);
        ctx->dScratch = nullptr;
        ctx->scratchCap = 0;
        PLT_CUDA(ctx, cudaMalloc(&ctx->dScratch, need));
        PLT_CUDA(ctx, cudaMemset(ctx->dScratch, 0, need));   // the schedule's control words start at zero
        ctx->scratchCap = need;
    }
    return pltLaunchBsdfBatch(ctx, p, ctx->dScratch, (cudaStream_t)stream);
}

plt_status plt_set_timing_events(plt_context* ctx, void* before_classify, void* before_shade, void* after_shade) {
    if (!ctx) return PLT_INVALID_ARG;
    ctx->timing[0] = before_classify;
    ctx->timing[1] = before_shade;
    ctx->timing[2] = after_shade;
    return PLT_OK;
}

plt_status plt_last_bounds_violation(const plt_context* ctx, uint32_t* out3) {
    if (!ctx || !out3) return PLT_INVALID_ARG;
    for (int k = 0; k < 3; ++k) out3[k] = ctx->boundsReport[k];
    return PLT_OK;
}

}  // extern "C"

plt_status pltLaunchBsdfBatch(plt_context* ctx, plt::BatchParams& p, void* scratch, cudaStream_t stream) {
    plt::pltBatchScratch(p, scratch);
    const cudaError_t e = plt::launchBsdfBatch(p, (int)p.q.hwss, ctx->numSMs, stream);
    return e == cudaSuccess ? PLT_OK : cudaFail(ctx, e);
}

plt_status plt::fillBatchParams(plt_context* ctx, const plt_bsdf_queries* q, const plt_bsdf_results* r, uint32_t ops,
                                plt::BatchParams* out, int* numSMs) {
    if (!ctx || !q || !r || !out || !numSMs) return PLT_INVALID_ARG;
    if (q->hwss < 1 || q->hwss > PLT_MAX_HWSS) return PLT_INVALID_ARG;
    if (q->hwss > 4 && q->hwss != 8) return PLT_NOT_SUPPORTED;
    if (ops == 0 || (ops & ~0xFu)) return PLT_INVALID_ARG;
    const plt_status ds = pltCheckDevice(ctx);
    if (ds != PLT_OK) return ds;
    if (q->n > 0) {
        if (!q->material || !q->v || !q->w || !q->wavelengths || !q->stokes || !q->coherence) return PLT_INVALID_ARG;
        if (ctx->nMats == 0) return PLT_INVALID_ARG;
        const void* ins[] = {q->material, q->v, q->w, q->lobe, q->wavelengths, q->stokes, q->coherence, q->beam_t};
        for (const void* ptr : ins)
            if (ptr && !aligned16(ptr)) return PLT_INVALID_ARG;
        const void* outs[] = {r->stokes, r->coherence, r->beam_t, r->pdf, r->lambda_pdf, r->sample_wo, r->sample_pdf,
                              r->sample_weight, r->sample_lobe, r->sample_valid};
        for (const void* ptr : outs)
            if (ptr && !aligned16(ptr)) return PLT_INVALID_ARG;
    }
    plt::BatchParams p{};
    p.q = *q;
    p.r = *r;
    p.ops = ops;
    p.mats = ctx->dMats;
    p.matType = ctx->dMatType;
    p.nMats = ctx->nMats;
    p.profiles = ctx->dProfiles;
    p.nProfiles = ctx->nProfiles;
    p.flags = ctx->opt.flags;
    p.status = ctx->dStatus;
    for (int i = 0; i < 3; ++i) p.timing[i] = ctx->timing[i];
    p.launch = &ctx->shadeLaunch;
    p.copyPolls = (ctx->opt.flags & PLT_OPTION_FAULT_COPY_WAIT) ? 0u : (1u << 22);
    *out = p;
    *numSMs = ctx->numSMs;
    return PLT_OK;
}

extern "C" {

plt_status plt_bsdf_eval(plt_context* c, const plt_bsdf_queries* q, const plt_bsdf_results* r, void* s) { return plt_bsdf_batch(c, q, r, PLT_OP_EVAL, s); }
plt_status plt_bsdf_pdf(plt_context* c, const plt_bsdf_queries* q, const plt_bsdf_results* r, void* s) { return plt_bsdf_batch(c, q, r, PLT_OP_PDF, s); }
plt_status plt_bsdf_sample(plt_context* c, const plt_bsdf_queries* q, const plt_bsdf_results* r, void* s) { return plt_bsdf_batch(c, q, r, PLT_OP_SAMPLE, s); }
plt_status plt_bsdf_lambda_pdf(plt_context* c, const plt_bsdf_queries* q, const plt_bsdf_results* r, void* s) { return plt_bsdf_batch(c, q, r, PLT_OP_LAMBDA_PDF, s); }

static plt_status traceCommon(plt_context* ctx, const plt_rays* rays, const plt_hits* hits, uint32_t* occluded, bool any, void* stream) {
    const plt::NvtxRange range(any ? "trace_any" : "trace_closest");
    if (!ctx || !rays) return PLT_INVALID_ARG;
    const plt_status ds = pltCheckDevice(ctx);
    if (ds != PLT_OK) return ds;
    if (ctx->geometryDirty) {
        const plt_status s = pltUploadScenes(ctx);
        if (s != PLT_OK) return s;
    }
    if (!ctx->dNodes) return PLT_INVALID_ARG;  // no scene
    if (rays->n == 0) return PLT_OK;
    if (!rays->origin || !rays->dir) return PLT_INVALID_ARG;
    if (any ? !occluded : (!hits || !hits->prim)) return PLT_INVALID_ARG;
    plt::TraceParams p{};
    p.n = rays->n;
    p.origin = rays->origin;
    p.dir = rays->dir;
    p.tmin = rays->tmin;
    p.tmax = rays->tmax;
    p.nodes = ctx->dNodes;
    p.tris = ctx->dTris;
    if (!any) {
        p.prim = hits->prim;
        p.t = hits->t;
        p.bary = hits->bary;
    }
    p.occluded = occluded;
    p.stats = reinterpret_cast<unsigned long long*>(rays->stats);
    p.status = ctx->dStatus;
    p.stackCap = (ctx->opt.flags & PLT_OPTION_FAULT_SHORT_STACK) ? 2 : 1 << 30;
    const cudaError_t e = plt::launchTrace(p, any, ctx->numSMs, (cudaStream_t)stream);
    return e == cudaSuccess ? PLT_OK : cudaFail(ctx, e);
}

plt_status plt_trace_closest(plt_context* ctx, const plt_rays* rays, const plt_hits* hits, void* stream) {
    return traceCommon(ctx, rays, hits, nullptr, false, stream);
}
plt_status plt_trace_any(plt_context* ctx, const plt_rays* rays, uint32_t* occluded, void* stream) {
    return traceCommon(ctx, rays, nullptr, occluded, true, stream);
}
plt_status plt_scene_stats(const plt_context* ctx, uint32_t* out4) {
    if (!ctx || !out4) return PLT_INVALID_ARG;
    out4[0] = ctx->bvhStats.nodes;
    out4[1] = ctx->bvhStats.leaves;
    out4[2] = ctx->bvhStats.maxDepth;
    out4[3] = ctx->nTris;
    return PLT_OK;
}

// Synchronises the stream and converts the device status word of the context (accumulated by
// every launch since the last check) into a status, then clears it.
plt_status plt_check_status(plt_context* ctx, void* stream) {
    if (!ctx) return PLT_INVALID_ARG;
    uint32_t w[plt::kStatusWords] = {};
    PLT_CUDA(ctx, cudaStreamSynchronize((cudaStream_t)stream));
    PLT_CUDA(ctx, cudaMemcpy(w, ctx->dStatus, sizeof(w), cudaMemcpyDeviceToHost));
    PLT_CUDA(ctx, cudaMemset(ctx->dStatus, 0, sizeof(w)));
    const uint32_t st = w[0];
    if (st & plt::kStatusBoundsViolation) {
        for (int k = 0; k < 3; ++k) ctx->boundsReport[k] = w[1 + k];
        return PLT_BOUNDS_VIOLATION;
    }
    if (st & (plt::kStatusCopyTimeout | plt::kStatusStackOverflow)) return PLT_QUEUE_TIMEOUT;
    if (st & (plt::kStatusBadMaterialId | plt::kStatusUnknownType)) return PLT_BAD_MATERIAL;
    if (st & plt::kStatusNanInput) return PLT_NAN_INPUT;
    return PLT_OK;
}

}  // extern "C"
