// Internal interface between the C-ABI host code and the CUDA kernels of libplt_gb300.so.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/plt_gb300.h"

namespace pltdev {
struct DevMaterial;
struct DevProfile;
}  // namespace pltdev

namespace plt {

// device status word bits (read back by plt_check_status)
constexpr uint32_t kStatusBadMaterialId = 0x1u;
constexpr uint32_t kStatusNanInput = 0x2u;
constexpr uint32_t kStatusUnknownType = 0x4u;
constexpr uint32_t kStatusCopyTimeout = 0x8u;
constexpr uint32_t kStatusStackOverflow = 0x10u;
constexpr uint32_t kStatusBoundsViolation = 0x20u;   // PLT_BOUNDS_CHECK builds: an index outside its buffer
// The context's device status block: [0] the status bits above; [1..3] the first bounds violation
// of a PLT_BOUNDS_CHECK build (site, index, bound).
constexpr uint32_t kStatusWords = 4;

// One batch of ray queries against the context's BVH (device pointers).
struct TraceParams {
    uint32_t n;
    const float* origin;          // [3][n]
    const float* dir;             // [3][n]
    const float* tmin;            // [n] or null
    const float* tmax;            // [n] or null
    const void* nodes;            // BvhNode[]
    const float4* tris;           // 3 float4 per triangle in leaf order; v0.w holds the triangle id bits
    uint32_t* prim;               // closest hit: [n]
    float* t;                     // closest hit: [n] or null
    float* bary;                  // closest hit: [2][n] or null
    uint32_t* occluded;           // any hit: [n]
    unsigned long long* stats;    // [2] node visits, triangle tests, or null
    uint32_t* status;
    int32_t stackCap;             // traversal stack entries (the full depth; 2 under PLT_OPTION_FAULT_SHORT_STACK)
};
cudaError_t launchTrace(const TraceParams& p, bool any, int numSMs, cudaStream_t stream);

// Resident shade-kernel CTAs per SM at a dynamic shared-memory size, per hero-wavelength count
// (index H).  Each context keeps its own, so contexts used from different host threads share no
// mutable launch state.
struct ShadeLaunchCache {
    size_t smem[9];
    int blocks[9];
    int classifyBlocks[9];   // resident classify CTAs per SM (0: not yet queried)
};

struct BatchParams {
    plt_bsdf_queries q;
    plt_bsdf_results r;
    uint32_t ops;
    const pltdev::DevMaterial* mats;
    const uint8_t* matType;
    uint32_t nMats;
    const pltdev::DevProfile* profiles;
    uint32_t nProfiles;
    uint32_t flags;
    uint32_t* status;
    // scratch (bsdfScratchBytes): the per-tile sort permutation (kBatchTile 16-bit local indices
    // per tile, sorted by material type then lobe class), each tile's material-type ranges in it
    // (kTypeSlots + 1 offsets per tile), the schedule's control words and the SM -> type table
    uint16_t* perm;
    uint16_t* tileTypeOff;
    uint32_t* ctrl;            // BatchCtrl words (see plt_bsdf_kernel.cuh)
    uint8_t* smType;           // [kMaxSmIds] material type each SM starts on
    uint32_t unitQueries;      // target queries per work unit (a multiple of 32)
    uint32_t smallBatch;       // at most kSmallBatchTiles tiles: not classified (see plt_bsdf_kernel.cuh)
    uint32_t copyPolls;        // poll budget of the spectral-table copy wait (0 under PLT_OPTION_FAULT_COPY_WAIT)
    float typeCost[16];        // relative cost per query of each material type (the schedule's SM shares)
    // optional cudaEvent_t handles recorded on the launch stream before the classify kernel,
    // between the two kernels and after the shade kernel (per-kernel timing); null = not recorded
    void* timing[3];
    ShadeLaunchCache* launch;  // host-side occupancy cache of the calling context (not read on the device)
};

// PLTPT render pass (sample + solve).  Per-material property word (matProps.x):
// bits 0-3 BSDFProperties flags, 8-15 getLobes() bits, 16 double-sided, 17 alpha == 0;
// matProps.y = emission profile id.
constexpr uint32_t kPropEmissive = 0x1u, kPropTransmissive = 0x2u, kPropMwReflective = 0x4u, kPropMwTransmissive = 0x8u;
constexpr uint32_t kPropDoubleSided = 1u << 16, kPropAlphaZero = 1u << 17;
// option bits of PtParams.opt
constexpr uint32_t kPtHwssMis = 0x1u, kPtUseDirect = 0x2u, kPtUseEmissive = 0x4u, kPtDoNee = 0x8u, kPtDoMis = 0x10u,
                   kPtDoRR = 0x20u, kPtPerTileSg = 0x40u, kPtImportanceEmit = 0x80u, kPtDoMnee = 0x100u,
                   kPtLearned = 0x200u, kPtUseEnv = 0x400u, kPtUseAnalytic = 0x800u,
                   kPtUniformEmissive = 0x1000u, kPtTinySg = 0x2000u, kPtAlphaMask = 0x4000u;
// solve-order sort keys per path length: 16 first-hit material types x 4 second-hit material groups
constexpr uint32_t kSolveKeysPerLength = 64;
// bytes reserved per deferred manifold walk (the device task structure is checked against it)
constexpr size_t kMneeTaskBytes = 320;
// bytes reserved per deferred forward replay (a sourced beam at up to 8 wavelengths and its vertex)
constexpr size_t kReplayTaskBytes = 288;
// replay-order sort keys: vertices to evaluate (0..15) x material type of the first one (16)
constexpr uint32_t kSegKeys = 16;         // segment shading order: the hit's material type, 15 for a miss
constexpr uint32_t kSegSortWords = 48;    // per segment: kSegKeys counts, kSegKeys cursors, the work counter
constexpr uint32_t kReplayKeys = 256;

// One scene of a render: its BVH root in the combined node array, its light range in the combined
// light arrays (the power sampler's table holds scene-local indices), its camera, image size, the
// first path of its pixels in the frame's path range, and its output image.
struct PtScene {
    plt_camera cam;
    uint32_t width, height, pixelBase, root;
    uint32_t lightBase, nLights;
    float invWeightsSum;
    uint32_t activeBase, nActive; // the scene's active lights (flux > 0) in PtParams.lightActive
    uint32_t pad;
    float* out;                   // [height][width][4]
};

// The environment light of a render (EnvMap.slang, EnvMapSampler.slang): an RGB lat-long map
// (float4 texels, [height][width]) filtered bilinearly with U wrapped and V clamped, scaled by
// intensity x tint; and the sampler's hierarchical importance map over the equal-area octahedral
// parameterisation (imp: the mip chain concatenated, level 0 of impDim x impDim first, level k at
// mipOff[k]; level impBaseMip is the 1x1 average).  toWorld / toLocal: row-major rotations.
constexpr uint32_t kEnvImportanceDim = 512, kEnvImportanceSpp = 64, kEnvMaxMips = 16;
struct EnvDev {
    const float4* tex;
    uint32_t width, height;
    const float* imp;
    uint32_t impDim, impBaseMip;
    uint32_t mipOff[kEnvMaxMips];
    float toWorld[9], toLocal[9];
    float scale[3];               // intensity * tint
};

// An analytic light on the device (LightData): the position, direction and spot parameters, the
// distant light's subtended angle, the area light's surface area and model-to-world transform (rows
// of a 3x4) with the inverse-transpose of its 3x3 part (normals), and the area lights' constant
// world normal normalize(transMatIT (0, 0, 1)).
struct AnalyticLightDev {
    float pos[3];
    uint32_t type;
    float dir[3];
    uint32_t spectrumId;
    float openingAngle, cosOpeningAngle, penumbraAngle, cosSubtendedAngle;
    float surfaceArea;
    float nrm[3];
    float xf[12];
    float xfIT[9];
    float pad[3];
};

// Launch shape of a render (chosen by plt_render_tune; zeros: defaults): paths per wave (0 = all
// paths of the frame in one wave) and blocks of 128 per SM for the segment, solve and
// manifold-walk kernels (0 = the occupancy limit).
struct PtLaunch {
    uint32_t waveCap;
    uint32_t segBlocksPerSM, solveBlocksPerSM, walkBlocksPerSM;
    uint32_t noLengthSort;        // solve-pass order: 0 sorted by length for waves >= 2^18 paths, 1 path order, 2 always sorted
};

struct PtParams {
    // scene
    const void* nodes;
    const float4* tris;
    const float* pos;             // [nv][3]
    const float* nrm;             // [nv][3]
    const float* tan;             // [nv][4] or null
    const uint32_t* idx;          // [nt][3]
    const uint32_t* triMat;       // [nt]
    const uint32_t* triInst;      // [nt] geometry instance (manifold re-projection)
    uint32_t nTris;
    const pltdev::DevMaterial* mats;
    const uint2* matProps;
    uint32_t nMats;
    const pltdev::DevProfile* profiles;
    const float* profileIcdf;     // [nProfiles][128]
    uint32_t nProfiles;
    // light collection
    const float* lightPos;        // [nl][9]
    const float* lightNrm;        // [nl][3]
    const float* lightArea;       // [nl]
    const float* lightFlux;       // [nl]
    const uint2* alias;           // [nl]
    const uint32_t* primToLight;  // [nt]
    const uint32_t* lightEmission;// [nl] emission profile id
    const uint32_t* lightActive;  // active lights (flux > 0) of every scene, global light indices
    // scenes of this render (one for plt_render, several for plt_render_scenes)
    const PtScene* scenes;
    uint32_t nScenes;
    // options
    uint32_t maxBounces, tileSize, hwss, opt, flags;
    float sourcingArea, maxBeamOmega;
    uint32_t mneeMaxOccluders, mneeMaxIterations;
    float mneeThreshold;
    uint32_t debugView;           // PLT_DEBUG_VIEW_* (0: none; manifold walks then run inline in the solve kernel)
    float debugIntensity;
    // paths: the frame's paths of all views are processed in waves of at most `npix` paths (the
    // plane stride of the path state and bounce records); this wave holds paths
    // [pidBase, pidBase + nWave) of the frame's nTotal
    uint32_t npix, nWave, pidBase, nTotal;
    const uint32_t* frameDev;     // the frame index (device word: one recorded launch sequence serves every frame)
    // path state of the sample pass
    uint32_t* sg;                 // [4][npix]
    float* org;                   // [3][npix]
    float* dir;                   // [3][npix]
    float* wl;
    float* weight;
    float* pdf;
    float* thp;
    float* lndp;
    uint32_t* pflags;
    uint32_t* plen;
    uint32_t* queue0;             // [npix]
    uint32_t* queue1;             // [npix]
    uint32_t* segPrim;            // [npix] closest hit of each queue slot of the segment (ptSegTraceKernel), or null:
    float* segBary;               // [2][npix]   the segment kernels then trace inline
    uint32_t* segOrder;           // [npix] the segment's queue slots sorted by the hit's material type, or null
    uint32_t* segSort;            // [maxBounces + 1][kSegSortWords]: key counts, cursors, the shade kernel's work counter
    uint32_t* qcount;             // [maxBounces + 2]
    uint32_t* lenCount;           // [16 (maxBounces + 1)] paths per solve-order key (length, first-hit type)
    uint32_t* lenCursor;          // [16 (maxBounces + 1)]
    const uint32_t* order;        // solve-pass path order (longest paths first), or null = path order
    // bounce buffer, planes [maxBounces + 1][npix] (two planes per bounce for bary / encoded wi)
    uint32_t* bPrim;
    float* bBary;
    float* bEw;
    uint32_t* bLobe;
    uint32_t* bFlags;
    float* bContrib;
    float* bLndp;
    // learned MIS proposal (kPtLearned)
    const void* propNet;          // bf16 parameters
    const float4* matFeat;        // [nMats] (roughness, pitch feature, class, enabled)
    float propProb;               // probability of the learned strategy at a proposal vertex
    float* wpss;                  // [npix] product of primary-sample MIS densities, or null
    // deferred manifold walks of the solve pass (null: walks run inline)
    void* mneeTasks;              // [mneeCap] tasks of kMneeTaskBytes
    uint32_t mneeCap;
    uint32_t* mneeCount;
    uint32_t* mneeSort;           // [32] walk-order key counts and cursors
    uint32_t* mneeOrder;          // [mneeCap] walk order of the tasks (sorted by occluder count and material), or null
    // deferred forward replays of the solve pass (null: replays run inline)
    void* replayTasks;            // [replayCap] tasks of kReplayTaskBytes
    uint32_t replayCap;
    uint32_t* replayCount;
    uint32_t* replaySort;         // [2 kReplayKeys + 1] replay-order key counts and cursors, the replay work counter
    uint32_t* replayOrder;        // [replayCap] replay order (sorted by vertex count and first material)
    // environment light (kPtUseEnv) and analytic lights (kPtUseAnalytic)
    EnvDev env;
    const AnalyticLightDev* alights;
    uint32_t nALights;
    // outputs
    double* accum;                // [npix][3]
    unsigned long long* stats;    // [4] bounces recorded, shadow rays, forward BSDF evaluations, traversal bytes
    uint32_t* status;
};
cudaError_t launchRenderFrame(const PtParams& p, const PtLaunch& L, int numSMs, cudaStream_t stream);
cudaError_t launchSetFrame(uint32_t* frameDev, uint32_t frame, bool advance, cudaStream_t stream);
// Builds the environment sampler's importance map (base level, then the mips) from env.tex into
// env.imp (plt_envmap.cu).
cudaError_t launchEnvImportance(const EnvDev& env, cudaStream_t stream);
// Sampler queries for tests: per query i, sample(u[i]) and eval / evalPdf of dirs[i] (plt_envmap.cu).
cudaError_t launchEnvQuery(const EnvDev& env, const float* u, const float* dirs, uint32_t n, float* out, cudaStream_t stream);

constexpr int kBatchThreads = 256;     // classify CTA
constexpr int kBatchItems = 8;
constexpr int kBatchTile = kBatchThreads * kBatchItems;
constexpr int kShadeThreads = 128;     // shade CTA
// Resident shade CTAs per SM the register allocation must allow.  One wavelength per beam: 4 (16
// warps, at most 128 registers; the natural allocation of the BSDF units' code is 154, which gives
// 3): 0.563 against 0.620 ms on the 2^22 mixed batch, and configuration 0's 2,048 warps fit in one
// wave (14.4 against 16.3 us).  More wavelengths: 3 (up to 170 registers; 4 spills 60 to 1,400
// bytes per thread).
#ifndef PLT_SHADE_MIN_BLOCKS
#define PLT_SHADE_MIN_BLOCKS 3
#endif
#ifndef PLT_SHADE_MIN_BLOCKS_H1
#define PLT_SHADE_MIN_BLOCKS_H1 4
#endif
template <int H> constexpr int shadeMinBlocks() { return H == 1 ? PLT_SHADE_MIN_BLOCKS_H1 : PLT_SHADE_MIN_BLOCKS; }

// Material types of the schedule (plt_material_type ids 0..15; invalid ids land in their own slot).
constexpr uint32_t kTypeSlots = 16;
// Upper bound of the %smid values of the SM -> type table.
constexpr uint32_t kMaxSmIds = 256;
constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
// Scratch layout of a batch of n queries: control words | SM table | permutation | tile type offsets.
// The control words come first so that their place does not depend on n: a scratch buffer reused
// for batches of any size keeps them.
constexpr size_t bsdfPermBytes(uint32_t n) { return align256(((size_t)n + kBatchTile - 1) / kBatchTile * kBatchTile * sizeof(uint16_t)); }
constexpr size_t bsdfTileOffBytes(uint32_t n) {
    return align256(((size_t)n + kBatchTile - 1) / kBatchTile * (kTypeSlots + 1) * sizeof(uint16_t));
}
constexpr size_t kBsdfCtrlBytes = 1024;
// scratch bytes plt_bsdf_batch needs for n queries; the control words must be zero before the first
// batch (they are left zero by every batch)
constexpr size_t bsdfScratchBytes(uint32_t n) { return bsdfPermBytes(n) + bsdfTileOffBytes(n) + kBsdfCtrlBytes + kMaxSmIds; }

// Points a batch's scratch fields into `scratch` (bsdfScratchBytes(p.q.n) bytes, 256-byte aligned).
inline void pltBatchScratch(BatchParams& p, void* scratch) {
    char* b = static_cast<char*>(scratch);
    p.ctrl = reinterpret_cast<uint32_t*>(b);
    b += kBsdfCtrlBytes;
    p.smType = reinterpret_cast<uint8_t*>(b);
    b += kMaxSmIds;
    p.perm = reinterpret_cast<uint16_t*>(b);
    b += bsdfPermBytes(p.q.n);
    p.tileTypeOff = reinterpret_cast<uint16_t*>(b);
}

// Validates a plt_bsdf_batch call and fills every BatchParams field except the scratch pointers
// (perm, tileTypeOff, ctrl, smType); also returns the SM count for the launch.  No allocation.  Returns
// PLT_INVALID_ARG when the calling thread's current device is not the context's device.
plt_status fillBatchParams(plt_context* ctx, const plt_bsdf_queries* q, const plt_bsdf_results* r, uint32_t ops,
                           BatchParams* out, int* numSMs);

// Launches the fused BSDF batch kernel (templated on the hero-wavelength count).
cudaError_t launchBsdfBatch(const BatchParams& p, int hwss, int numSMs, cudaStream_t stream);

}  // namespace plt
