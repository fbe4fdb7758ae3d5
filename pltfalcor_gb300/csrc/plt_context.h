// The library context (opaque to callers): device tables, scene, render-pass buffers, and the
// host copies the render pass's light collection is built from.
#pragma once

#include <cuda_runtime.h>

#include <vector>

#include "plt_bvh.h"
#include "plt_host.h"
#include "plt_internal.h"

struct plt_host_pipeline;   // plt_bsdf_batch_host's staging slots, copy streams and events (plt_host_batch.cpp)

// One scene of the context's scene set, kept on the host: its BVH (scene-local node and triangle
// indices), triangles in leaf order, and its shading attributes.  The device holds all scenes
// concatenated (pltUploadScenes).
struct plt_scene_host {
    std::vector<plt::BvhNode> nodes;
    std::vector<float4> tris;          // 3 per triangle, leaf order; .w of the first = local triangle id
    std::vector<float> pos, nrm, tan;  // tan empty: no tangents
    std::vector<uint32_t> idx, triMat, triInst;
    uint32_t nVerts = 0, nTris = 0;
    plt::BvhBuildStats stats{};
    bool shaded = false;
};
// A scene's place in the combined device arrays.
struct plt_scene_slot {
    uint32_t root = 0, triBase = 0, lightBase = 0, nLights = 0;
    float invWeightsSum = 0.f;
    uint32_t activeBase = 0, nActive = 0;   // the scene's active (flux > 0) lights in dLightActive
};

struct plt_context {
    int device = 0;
    int numSMs = 0;
    plt_options opt{};
    pltdev::DevMaterial* dMats = nullptr;
    uint8_t* dMatType = nullptr;
    uint32_t nMats = 0, capMats = 0;
    pltdev::DevProfile* dProfiles = nullptr;
    uint32_t nProfiles = 0, capProfiles = 0;
    uint32_t* dStatus = nullptr;
    void* dScratch = nullptr;     // batch scratch (sort permutation + work counter), grown on demand
    size_t scratchCap = 0;
    // scene
    plt::BvhNode* dNodes = nullptr;
    float4* dTris = nullptr;      // 3 float4 per triangle, leaf order
    uint32_t* dTriMaterial = nullptr;
    uint32_t nTris = 0;
    plt::BvhBuildStats bvhStats{};
    int lastCudaError = 0;
    uint32_t boundsReport[3] = {0u, 0u, 0u};   // the last reported bounds violation (site, index, bound)
    void* timing[3] = {nullptr, nullptr, nullptr};   // cudaEvent_t handles recorded by plt_bsdf_batch
    plt::ShadeLaunchCache shadeLaunch = {{(size_t)-1, (size_t)-1, (size_t)-1, (size_t)-1, (size_t)-1, (size_t)-1, (size_t)-1,
                                          (size_t)-1, (size_t)-1},
                                         {},
                                         {}};

    // host copies for the render pass (light collection, material properties)
    std::vector<plt_spectral_profile> hProfiles;
    std::vector<plt_material_record> hMats;
    std::vector<pltdev::DevMaterial> hDevMats;
    std::vector<plt_scene_host> scenes;   // the scene set (plt_set_scene: one scene)
    std::vector<plt_scene_slot> slots;    // each scene's root, triangle and light ranges on the device
    bool geometryDirty = false, shadingDirty = false;
    uint32_t nVerts = 0;                  // vertices of the last scene set (plt_set_scene_shading checks it)
    plt::PtScene* dScenes = nullptr;      // per-render scene table
    uint32_t scenesCap = 0;
    float* dProfileIcdf = nullptr;   // [nProfiles][128]
    uint2* dMatProps = nullptr;      // [nMats]
    float* dPos = nullptr;           // [nVerts][3]
    uint32_t* dIdx = nullptr;        // [nTris][3]
    float* dNrm = nullptr;           // [nVerts][3]
    float* dTan = nullptr;           // [nVerts][4] or null
    uint32_t* dTriInst = nullptr;    // [nTris] geometry instance
    bool shadingReady = false;
    // light collection + power sampler
    float* dLightPos = nullptr;
    float* dLightNrm = nullptr;
    float* dLightArea = nullptr;
    float* dLightFlux = nullptr;
    uint2* dAlias = nullptr;
    uint32_t* dPrimToLight = nullptr;
    uint32_t* dLightEmission = nullptr;
    uint32_t* dLightActive = nullptr;   // active light triangles (flux > 0) of every scene, global light indices
    uint32_t nLights = 0;
    float invWeightsSum = 0.f;
    // render-pass buffers (one allocation, sized for ptNpix paths and ptMaxB bounces)
    void* dPt = nullptr;
    size_t ptBytes = 0;
    void* dPtMix = nullptr;       // per-path primary-sample MIS density products (learned renders)
    size_t ptMixBytes = 0;
    void* dMneeTasks = nullptr;   // deferred manifold walks of the solve pass
    size_t mneeBytes = 0;
    void* dReplayTasks = nullptr; // deferred forward replays of the solve pass, then their order
    size_t replayBytes = 0;
    uint32_t ptNpix = 0, ptMaxB = 0;
    uint64_t lastPaths = 0;       // paths of all views in the last render
    double* dAccum = nullptr;     // [paths of all views][3] frame accumulation
    uint32_t accumCap = 0;
    plt::PtLaunch launch{};       // launch shape (plt_render_tune; zeros = defaults)
    uint32_t* dFrame = nullptr;   // frame index word of the render kernels
    void* capStream = nullptr;    // cudaStream_t the frame graph is recorded on
    void* graphExec = nullptr;    // cudaGraphExec_t of one frame's launch sequence
    std::vector<unsigned char> graphKey;   // the parameters it was recorded with
    plt::PtParams pt{};
    unsigned long long* dPtStats = nullptr;
    // learned MIS proposal: FP32 master weights, Adam moments, BF16 copy, gradient, loss;
    // per-material features (roughness, pitch, class, enabled) and the enabled-material list
    float* dPropParams = nullptr;
    float* dPropM = nullptr;
    float* dPropV = nullptr;
    void* dPropBf16 = nullptr;
    float* dPropGrad = nullptr;
    float* dPropLoss = nullptr;
    uint32_t propStep = 0;
    bool propReady = false;
    float4* dMatFeat = nullptr;
    uint32_t* dPropEnabled = nullptr;
    uint32_t nPropEnabled = 0;
    void* dPropBatch = nullptr;      // training batch (features, targets, weights)
    uint32_t propBatchCap = 0;
    // environment light: the map (float4 texels) and the sampler's importance mip chain
    float4* dEnvTex = nullptr;
    size_t envTexCap = 0;
    float* dEnvImp = nullptr;
    plt::EnvDev env{};
    bool hasEnv = false;
    // analytic lights
    plt::AnalyticLightDev* dALights = nullptr;
    uint32_t nALights = 0;
    plt_host_pipeline* hostPipe = nullptr;
};

// PLT_OK when the calling thread's current CUDA device is the one the context was created on; a
// context's buffers, kernels' occupancy and scratch belong to that device, so every launching entry
// point refuses (PLT_INVALID_ARG) to run on another one.
inline plt_status pltCheckDevice(plt_context* ctx) {
    int dev = -1;
    const cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) {
        ctx->lastCudaError = (int)e;
        return PLT_CUDA_ERROR;
    }
    return dev == ctx->device ? PLT_OK : PLT_INVALID_ARG;
}

// Points the batch's sort permutation and work counter into `scratch` (at least
// bsdfScratchBytes(p.q.n) bytes) and launches the classify + shade kernels on `stream`
// (plt_capi.cpp).
plt_status pltLaunchBsdfBatch(plt_context* ctx, plt::BatchParams& p, void* scratch, cudaStream_t stream);

// Frees the render-pass state of a context (plt_render.cpp).
void pltReleaseRenderState(plt_context* ctx);
// Material property word for the render pass (plt_render.cpp).
uint2 pltMaterialProps(const plt_material_record& r, const pltdev::DevMaterial& d);
// Learned-proposal features of a material: (roughness, pitch feature, class, enabled) (plt_proposal.cpp).
float4 pltProposalFeatures(const plt_material_record& r, const pltdev::DevMaterial& d);
// Frees the learned-proposal state (plt_proposal.cpp).
void pltReleaseProposal(plt_context* ctx);

// Frees plt_bsdf_batch_host's pipeline (plt_host_batch.cpp).
void pltReleaseHostPipeline(plt_context* ctx);
// Frees the environment light (plt_scenes.cpp).
void pltReleaseEnv(plt_context* ctx);
// Uploads the scene set if it changed (geometry, shading, light collections); plt_scenes.cpp.
plt_status pltUploadScenes(plt_context* ctx);
