// Host side of the PLTPT render pass: per-material property words, the emissive-triangle light
// collection with the power sampler's alias table, render-buffer management and the frame loop.
// Paths cited are inside ssteinberg/PLTFalcor.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

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

template <class T> plt_status upload(plt_context* ctx, T*& dst, const T* src, size_t count) {
    cudaFree(dst);
    dst = nullptr;
    if (count == 0) return PLT_OK;
    PLT_CUDA(ctx, cudaMalloc(&dst, sizeof(T) * count));
    PLT_CUDA(ctx, cudaMemcpy(dst, src, sizeof(T) * count, cudaMemcpyHostToDevice));
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
    // the counters: per-segment queue lengths, the manifold-walk count, the solve-order keys per
    // length (counts, cursors), the walk-order keys, the replay count, the replay-order keys and
    // the replay kernel's work counter
    const size_t nCounters = nb + 2 + 2 * (size_t)plt::kSolveKeysPerLength * nb + 32 + 1 + 2 * (size_t)plt::kReplayKeys + 1 +
                             (size_t)plt::kSegSortWords * nb;
    const size_t pathBytes = al(4 * n * 4) + 2 * al(3 * n * 4) + 5 * al(n * 4) + 2 * al(n * 4) + 2 * al(n * 4) + al(nCounters * 4) +
                             al(n * 4) + al(2 * n * 4) + al(n * 4);
    const size_t bounceBytes = 2 * al(nb * n * 4) * 2 + 5 * al(nb * n * 4);
    const size_t total = pathBytes + bounceBytes;
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
    // per-segment queue lengths, the manifold-walk task count, the path-length histogram and cursors
    P.qcount = (uint32_t*)take(nCounters * 4);
    P.mneeCount = P.qcount + nb + 1;
    P.lenCount = P.qcount + nb + 2;
    P.lenCursor = P.lenCount + plt::kSolveKeysPerLength * nb;
    P.mneeSort = P.lenCursor + plt::kSolveKeysPerLength * nb;
    P.replayCount = P.mneeSort + 32;
    P.replaySort = P.replayCount + 1;
    P.mneeOrder = P.queue1;   // free during the solve pass
    P.segPrim = (uint32_t*)take(n * 4);
    P.segBary = (float*)take(2 * n * 4);
    P.segOrder = (uint32_t*)take(n * 4);
    P.segSort = P.replaySort + 2 * plt::kReplayKeys + 1;
    P.bBary = (float*)take(2 * nb * n * 4);
    P.bEw = (float*)take(2 * nb * n * 4);
    P.bPrim = (uint32_t*)take(nb * n * 4);
    P.bLobe = (uint32_t*)take(nb * n * 4);
    P.bFlags = (uint32_t*)take(nb * n * 4);
    P.bContrib = (float*)take(nb * n * 4);
    P.bLndp = (float*)take(nb * n * 4);
    ctx->ptNpix = npix;
    ctx->ptMaxB = maxB;
    return PLT_OK;
}

}  // namespace

namespace plt {
cudaError_t launchResolve(const PtParams& p, uint32_t frames, int numSMs, cudaStream_t stream);
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
    if (ctx->graphExec) cudaGraphExecDestroy((cudaGraphExec_t)ctx->graphExec);
    if (ctx->capStream) cudaStreamDestroy((cudaStream_t)ctx->capStream);
    cudaFree(ctx->dFrame);
    void* ptrs[] = {ctx->dProfileIcdf, ctx->dMatProps, ctx->dPos, ctx->dIdx, ctx->dNrm, ctx->dTan, ctx->dTriInst, ctx->dLightPos, ctx->dLightNrm,
                    ctx->dLightArea, ctx->dLightFlux, ctx->dAlias, ctx->dPrimToLight, ctx->dLightEmission, ctx->dLightActive, ctx->dPt, ctx->dPtStats, ctx->dPtMix, ctx->dMneeTasks, ctx->dReplayTasks, ctx->dScenes, ctx->dAccum};
    for (void* p : ptrs) cudaFree(p);
}

namespace {

// One render of a set of views: per-view validation, the scene table, buffers for all views'
// paths, the frame loop and the per-view resolve.
plt_status renderViews(plt_context* ctx, const plt_render_view* views, uint32_t nViews, uint32_t frame_begin, uint32_t frame_count,
                       void* stream) {
    if (!ctx || !views || nViews == 0 || frame_count == 0) return PLT_INVALID_ARG;
    plt_status s = pltCheckDevice(ctx);
    if (s != PLT_OK) return s;
    s = pltUploadScenes(ctx);
    if (s != PLT_OK) return s;
    if (!ctx->shadingReady || ctx->nTris == 0 || ctx->nMats == 0) return PLT_INVALID_ARG;
    const plt_options& o = ctx->opt;
    if (o.hwss < 1 || (o.hwss > 4 && o.hwss != 8)) return PLT_NOT_SUPPORTED;   // 8: beyond the reference's 1-4
    if (o.mnee_max_occluders > 4) return PLT_NOT_SUPPORTED;
    if (o.max_bounces > 64) return PLT_NOT_SUPPORTED;
    if (o.debug_view > PLT_DEBUG_VIEW_MNEE_BOUNCES) return PLT_INVALID_ARG;
    if (o.debug_view == PLT_DEBUG_VIEW_ALBEDO || o.debug_view == PLT_DEBUG_VIEW_ROUGHNESS) return PLT_NOT_SUPPORTED;
    if (o.sample_generator > PLT_SAMPLE_GENERATOR_UNIFORM) return PLT_INVALID_ARG;
    const bool learned = o.learned_proposal != 0;
    if (learned && (!ctx->propReady || !ctx->dMatFeat || !(o.learned_proposal_prob > 0.f && o.learned_proposal_prob < 1.f)))
        return PLT_INVALID_ARG;
    std::vector<plt::PtScene> table(nViews);
    uint64_t npix64 = 0;
    for (uint32_t v = 0; v < nViews; ++v) {
        const plt_render_view& rv = views[v];
        if (rv.scene >= ctx->scenes.size() || !rv.out_rgba || ((uintptr_t)rv.out_rgba & 15u) != 0) return PLT_INVALID_ARG;
        const plt_scene_slot& sl = ctx->slots[rv.scene];
        plt::PtScene& S = table[v];
        std::memset(&S, 0, sizeof(S));
        S.cam = rv.camera;
        S.width = rv.width;
        S.height = rv.height;
        S.pixelBase = (uint32_t)npix64;
        S.root = sl.root;
        S.lightBase = sl.lightBase;
        S.nLights = sl.nLights;
        S.invWeightsSum = sl.invWeightsSum;
        S.activeBase = sl.activeBase;
        S.nActive = sl.nActive;
        S.out = rv.out_rgba;
        npix64 += (uint64_t)rv.width * rv.height;
        if (npix64 > (1u << 26)) return PLT_NOT_SUPPORTED;
    }
    if (npix64 == 0) return PLT_OK;
    // views without pixels take no path range: drop them from the lookup table
    table.erase(std::remove_if(table.begin(), table.end(), [](const plt::PtScene& S) { return S.width == 0 || S.height == 0; }),
                table.end());
    const uint32_t total = (uint32_t)npix64;
    // paths per wave: the tuned cap, else the whole frame
    const plt::PtLaunch L = ctx->launch;
    const uint32_t npix = L.waveCap ? std::min(L.waveCap, total) : total;
    s = ensureRenderBuffers(ctx, npix, o.max_bounces);
    if (s != PLT_OK) return s;
    if (ctx->accumCap < total) {
        cudaFree(ctx->dAccum);
        ctx->dAccum = nullptr;
        ctx->accumCap = 0;
        PLT_CUDA(ctx, cudaMalloc(&ctx->dAccum, sizeof(double) * 3 * (size_t)total));
        ctx->accumCap = total;
    }
    const cudaStream_t st = (cudaStream_t)stream;
    if (ctx->scenesCap < table.size()) {
        cudaFree(ctx->dScenes);
        ctx->dScenes = nullptr;
        ctx->scenesCap = 0;
        PLT_CUDA(ctx, cudaMalloc(&ctx->dScenes, sizeof(plt::PtScene) * table.size()));
        ctx->scenesCap = (uint32_t)table.size();
    }
    PLT_CUDA(ctx, cudaMemcpyAsync(ctx->dScenes, table.data(), sizeof(plt::PtScene) * table.size(), cudaMemcpyHostToDevice, st));
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
    plt::PtParams& P = ctx->pt;
    P.scenes = ctx->dScenes;
    P.nScenes = (uint32_t)table.size();
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
    P.lightActive = ctx->dLightActive;
    P.maxBounces = o.max_bounces;
    P.tileSize = o.tile_size ? o.tile_size : 512;
    P.hwss = o.hwss;
    P.flags = o.flags;
    const bool nee = o.do_nee != 0;
    // light types: emissive geometry and the environment map, no analytic lights (PLTPT.cpp:230-232)
    P.opt = (o.hwss_do_mis ? plt::kPtHwssMis : 0u) | (o.use_direct_light ? plt::kPtUseDirect : 0u) |
            (o.use_emissive_lights && ctx->nLights ? plt::kPtUseEmissive : 0u) | (nee ? plt::kPtDoNee : 0u) |
            (nee && o.do_mis ? plt::kPtDoMis : 0u) | (o.do_russian_roulette ? plt::kPtDoRR : 0u) |
            (nee && o.nee_use_per_tile_sg ? plt::kPtPerTileSg : 0u) | (o.do_importance_sample_emitters ? plt::kPtImportanceEmit : 0u) |
            (nee && o.do_mnee ? plt::kPtDoMnee : 0u) | (learned ? plt::kPtLearned : 0u) |
            (o.use_env_light && ctx->hasEnv ? plt::kPtUseEnv : 0u) |
            (o.use_analytic_lights && ctx->nALights ? plt::kPtUseAnalytic : 0u) |
            (o.emissive_sampler == 0u ? plt::kPtUniformEmissive : 0u) |
            (o.sample_generator == PLT_SAMPLE_GENERATOR_TINY_UNIFORM ? plt::kPtTinySg : 0u) |
            (o.alpha_masking ? plt::kPtAlphaMask : 0u);
    P.env = ctx->env;
    P.alights = ctx->dALights;
    P.nALights = ctx->nALights;
    P.propNet = ctx->dPropBf16;
    P.matFeat = ctx->dMatFeat;
    P.propProb = o.learned_proposal_prob;
    P.wpss = learned ? static_cast<float*>(ctx->dPtMix) : nullptr;
    // deferred manifold walks: one task slot per path and frame (a fuller queue walks inline); a
    // debug view keeps them inline, where the path's debug colour is accumulated
    if (nee && o.do_mnee && o.debug_view == PLT_DEBUG_VIEW_NONE) {
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
    // deferred forward replays: 3/2 task slots per path and frame (beyond that they replay inline);
    // with a debug view they stay inline, where the path's debug colour is accumulated
    if (o.debug_view == PLT_DEBUG_VIEW_NONE && !(o.flags & PLT_OPTION_INLINE_REPLAY)) {
        const uint32_t cap = npix + npix / 2;
        const size_t bytes = (size_t)cap * (plt::kReplayTaskBytes + sizeof(uint32_t));
        if (ctx->replayBytes < bytes) {
            cudaFree(ctx->dReplayTasks);
            ctx->dReplayTasks = nullptr;
            ctx->replayBytes = 0;
            PLT_CUDA(ctx, cudaMalloc(&ctx->dReplayTasks, bytes));
            ctx->replayBytes = bytes;
        }
        P.replayTasks = ctx->dReplayTasks;
        P.replayCap = cap;
        P.replayOrder = reinterpret_cast<uint32_t*>(static_cast<char*>(ctx->dReplayTasks) + (size_t)cap * plt::kReplayTaskBytes);
    } else {
        P.replayTasks = nullptr;
        P.replayCap = 0;
        P.replayOrder = nullptr;
    }
    P.mneeMaxOccluders = o.mnee_max_occluders;
    P.mneeMaxIterations = o.mnee_max_iterations;
    P.mneeThreshold = o.mnee_solver_threshold;
    P.debugView = o.debug_view;
    P.debugIntensity = o.debug_view_intensity;
    P.sourcingArea = o.sourcing_area_from_emissive_geometry;
    P.maxBeamOmega = o.sourcing_max_beam_omega;
    P.npix = npix;
    P.nTotal = total;
    ctx->lastPaths = total;
    P.accum = ctx->dAccum;
    P.stats = ctx->dPtStats;
    P.status = ctx->dStatus;
    if (!ctx->dFrame) PLT_CUDA(ctx, cudaMalloc(&ctx->dFrame, sizeof(uint32_t)));
    P.frameDev = ctx->dFrame;
    P.pidBase = 0;
    P.nWave = 0;
    PLT_CUDA(ctx, cudaMemsetAsync(P.accum, 0, sizeof(double) * 3 * (size_t)total, st));
    PLT_CUDA(ctx, plt::launchSetFrame(ctx->dFrame, frame_begin, false, st));
    // one frame: the statistics reset, every wave's launch sequence, the frame-index advance
    auto enqueueFrame = [&](cudaStream_t s2) -> cudaError_t {
        plt::PtParams W = P;
        cudaError_t e = cudaMemsetAsync(ctx->dPtStats, 0, 4 * sizeof(unsigned long long), s2);
        for (uint32_t base = 0; e == cudaSuccess && base < total; base += npix) {
            W.pidBase = base;
            W.nWave = std::min(npix, total - base);
            e = plt::launchRenderFrame(W, L, ctx->numSMs, s2);
        }
        return e == cudaSuccess ? plt::launchSetFrame(ctx->dFrame, 0, true, s2) : e;
    };
    // The frame is recorded once per launch configuration as a CUDA graph and replayed per frame
    // (PLT_OPTION_NO_GRAPH launches it directly).
    bool replayed = false;
    if (!(o.flags & PLT_OPTION_NO_GRAPH)) {
        std::vector<unsigned char> key(sizeof(P) + sizeof(L) + sizeof(total));
        std::memcpy(key.data(), &P, sizeof(P));
        std::memcpy(key.data() + sizeof(P), &L, sizeof(L));
        std::memcpy(key.data() + sizeof(P) + sizeof(L), &total, sizeof(total));
        if (!ctx->graphExec || key != ctx->graphKey) {
            if (ctx->graphExec) cudaGraphExecDestroy((cudaGraphExec_t)ctx->graphExec);
            ctx->graphExec = nullptr;
            if (!ctx->capStream) PLT_CUDA(ctx, cudaStreamCreateWithFlags((cudaStream_t*)&ctx->capStream, cudaStreamNonBlocking));
            const cudaStream_t cs = (cudaStream_t)ctx->capStream;
            PLT_CUDA(ctx, cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed));
            const cudaError_t e1 = enqueueFrame(cs);
            cudaGraph_t g = nullptr;
            const cudaError_t e2 = cudaStreamEndCapture(cs, &g);
            cudaGraphExec_t x = nullptr;
            if (e1 == cudaSuccess && e2 == cudaSuccess && g && cudaGraphInstantiate(&x, g, 0) == cudaSuccess) {
                ctx->graphExec = x;
                ctx->graphKey = key;
            }
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();   // a failed recording falls back to direct launches
        }
        if (ctx->graphExec) {
            for (uint32_t f = 0; f < frame_count; ++f) PLT_CUDA(ctx, cudaGraphLaunch((cudaGraphExec_t)ctx->graphExec, st));
            replayed = true;
        }
    }
    if (!replayed)
        for (uint32_t f = 0; f < frame_count; ++f) PLT_CUDA(ctx, enqueueFrame(st));
    P.nWave = std::min(npix, total);
    PLT_CUDA(ctx, plt::launchResolve(P, frame_count, ctx->numSMs, st));
    return PLT_OK;
}

}  // namespace

extern "C" {

plt_status plt_render(plt_context* ctx, const plt_camera* camera, uint32_t width, uint32_t height, uint32_t frame_begin,
                      uint32_t frame_count, float* out_rgba, void* stream) {
    if (!ctx || !camera || !out_rgba || frame_count == 0) return PLT_INVALID_ARG;
    if (((uintptr_t)out_rgba & 15u) != 0) return PLT_INVALID_ARG;
    if ((uint64_t)width * height == 0) return PLT_OK;
    plt_render_view v;
    std::memset(&v, 0, sizeof(v));
    v.scene = 0;
    v.width = width;
    v.height = height;
    v.camera = *camera;
    v.out_rgba = out_rgba;
    const plt::NvtxRange range("render");
    return renderViews(ctx, &v, 1, frame_begin, frame_count, stream);
}

plt_status plt_render_scenes(plt_context* ctx, const plt_render_view* views, uint32_t n_views, uint32_t frame_begin, uint32_t frame_count,
                             void* stream) {
    const plt::NvtxRange range("render_scenes");
    return renderViews(ctx, views, n_views, frame_begin, frame_count, stream);
}

plt_status plt_set_launch_shape(plt_context* ctx, const plt_launch_shape* shape) {
    if (!ctx) return PLT_INVALID_ARG;
    ctx->launch = shape ? plt::PtLaunch{shape->wave_paths, shape->segment_blocks_per_sm, shape->solve_blocks_per_sm, shape->walk_blocks_per_sm,
                                        shape->path_order}
                        : plt::PtLaunch{};
    return PLT_OK;
}

plt_status plt_get_launch_shape(const plt_context* ctx, plt_launch_shape* shape) {
    if (!ctx || !shape) return PLT_INVALID_ARG;
    *shape = plt_launch_shape{ctx->launch.waveCap, ctx->launch.segBlocksPerSM, ctx->launch.solveBlocksPerSM, ctx->launch.walkBlocksPerSM,
                              ctx->launch.noLengthSort};
    return PLT_OK;
}

// Coordinate search over the launch shape on the caller's views: wave size first, then the
// blocks per SM of the segment, solve and manifold-walk kernels, each candidate timed (CUDA events
// on the caller's stream) over `frames` frames after one untimed frame that records its graph.
plt_status plt_render_tune(plt_context* ctx, const plt_render_view* views, uint32_t n_views, uint32_t frame, uint32_t frames,
                           plt_launch_shape* best, float* best_ms, void* stream) {
    const plt::NvtxRange range("render_tune");
    if (!ctx || !views || n_views == 0 || frames == 0) return PLT_INVALID_ARG;
    if (const plt_status ds = pltCheckDevice(ctx); ds != PLT_OK) return ds;
    uint64_t total = 0;
    for (uint32_t v = 0; v < n_views; ++v) total += (uint64_t)views[v].width * views[v].height;
    if (total == 0) return PLT_INVALID_ARG;
    const cudaStream_t st = (cudaStream_t)stream;
    cudaEvent_t e0, e1;
    PLT_CUDA(ctx, cudaEventCreate(&e0));
    PLT_CUDA(ctx, cudaEventCreate(&e1));
    uint32_t f = frame;
    // a candidate with a new wave size first renders one untimed frame (its buffers are sized
    // then); other candidates only re-record the frame graph, which the timed frames absorb
    uint32_t warmedWave = 0xFFFFFFFFu;
    auto timeShape = [&](const plt::PtLaunch& L, float& ms) -> plt_status {
        ctx->launch = L;
        plt_status s = PLT_OK;
        if (L.waveCap != warmedWave) {
            if ((s = renderViews(ctx, views, n_views, f, 1, stream)) != PLT_OK) return s;
            f += 1;
            warmedWave = L.waveCap;
        }
        if (cudaEventRecord(e0, st) != cudaSuccess) return PLT_CUDA_ERROR;
        if ((s = renderViews(ctx, views, n_views, f, frames, stream)) != PLT_OK) return s;
        f += frames;
        if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) return PLT_CUDA_ERROR;
        cudaEventElapsedTime(&ms, e0, e1);
        ms /= (float)frames;
        return PLT_OK;
    };
    plt::PtLaunch bestL{};
    float bestMs = 0.f;
    plt_status s = timeShape(bestL, bestMs);
    auto tryShape = [&](plt::PtLaunch L) {
        float ms = 0.f;
        if (s == PLT_OK && (s = timeShape(L, ms)) == PLT_OK && ms < bestMs) {
            bestMs = ms;
            bestL = L;
        }
    };
    for (uint32_t w : {1u << 22, 1u << 21, 1u << 20, 1u << 19, 1u << 18})
        if (w < total) tryShape(plt::PtLaunch{w, bestL.segBlocksPerSM, bestL.solveBlocksPerSM, bestL.walkBlocksPerSM, 0u});
    if (s == PLT_OK && bestL.waveCap != warmedWave) {   // the remaining candidates use the best wave size
        ctx->launch = bestL;
        s = renderViews(ctx, views, n_views, f, 1, stream);
        f += 1;
        warmedWave = bestL.waveCap;
    }
    for (uint32_t b : {2u, 4u}) tryShape(plt::PtLaunch{bestL.waveCap, b, bestL.solveBlocksPerSM, bestL.walkBlocksPerSM, 0u});
    for (uint32_t b : {1u}) tryShape(plt::PtLaunch{bestL.waveCap, bestL.segBlocksPerSM, b, bestL.walkBlocksPerSM, 0u});
    for (uint32_t b : {1u, 2u}) tryShape(plt::PtLaunch{bestL.waveCap, bestL.segBlocksPerSM, bestL.solveBlocksPerSM, b, 0u});
    for (uint32_t o : {1u, 2u}) tryShape(plt::PtLaunch{bestL.waveCap, bestL.segBlocksPerSM, bestL.solveBlocksPerSM, bestL.walkBlocksPerSM, o});
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    ctx->launch = bestL;
    if (s != PLT_OK) return s;
    if (best) *best = plt_launch_shape{bestL.waveCap, bestL.segBlocksPerSM, bestL.solveBlocksPerSM, bestL.walkBlocksPerSM, bestL.noLengthSort};
    if (best_ms) *best_ms = bestMs;
    return PLT_OK;
}


plt_status plt_render_counters(plt_context* ctx, uint64_t* out, uint32_t n) {
    if (!ctx || (n && !out)) return PLT_INVALID_ARG;
    unsigned long long h[4] = {0, 0, 0, 0};
    if (ctx->dPtStats) PLT_CUDA(ctx, cudaMemcpy(h, ctx->dPtStats, sizeof(h), cudaMemcpyDeviceToHost));
    const uint64_t v[5] = {ctx->lastPaths, h[0], h[1], h[2], h[3]};
    for (uint32_t i = 0; i < n && i < 5; ++i) out[i] = v[i];
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
