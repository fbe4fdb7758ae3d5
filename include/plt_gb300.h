/*
 * plt_gb300.h -- C ABI of the GB300-native PLT (physical light transport) hot path.
 *
 * One shared library (libplt_gb300.so) exports every function declared here.  The ABI uses
 * plain C types only: caller-owned pointers, sizes and status codes.  No exception crosses it.
 *
 * Conventions
 *  - Unless a comment says "host", every buffer pointer is a CUDA device pointer owned by the
 *    caller, 16-byte aligned, laid out as structure-of-arrays "planes": a field with C
 *    components over n queries is C consecutive planes of n values (component c of query i
 *    lives at [c*n + i]).
 *  - Every call returns a plt_status.  PLT_CUDA_ERROR carries the last cudaError_t, readable
 *    with plt_last_cuda_error().
 *  - Launches are asynchronous on the caller's stream (a cudaStream_t passed as void*;
 *    NULL = legacy default stream).  One context per host thread; distinct contexts are
 *    independent.
 *
 * Reference interfaces this ABI replaces (paths inside ssteinberg/PLTFalcor):
 *  - Material plugin: IMaterialInstance eval / sample / pdf / lambdaPdf
 *      Source/Falcor/Rendering/Materials/IMaterialInstance.slang:122-184, implemented per
 *      material in Source/Falcor/Rendering/Materials/PLT/PLT*BSDF.slang; material parameters
 *      packed by the PLT*Material.cpp host classes into BasicMaterialData
 *      (Source/Falcor/Scene/Material/BasicMaterialData.slang:63-85).
 *  - Spectral tables: SpectralProfile (BasicMaterialData.slang:43-54) built by
 *      SceneBuilder genSpectralProfile (Source/Falcor/Scene/SceneBuilder.cpp:911-960).
 *  - Render pass: PLTPT plugin create/execute (Source/RenderPasses/PLTPT/PLTPT.cpp:43-46,
 *      147-204, 357-499).
 */
#ifndef PLT_GB300_H
#define PLT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PLT_ABI_VERSION 5u
#define PLT_MAX_HWSS 8u                 /* hero wavelengths per beam (reference: <= 4, Utils/HWSS.slang:4-9) */
#define PLT_SPECTRAL_MAX_BINS 128u      /* SpectralProfile::kMaxBins */
#define PLT_NO_SPECTRAL_PROFILE 0xFFFFFFFFu

typedef enum plt_status {
    PLT_OK = 0,
    PLT_INVALID_ARG = 1,
    PLT_OOM = 2,
    PLT_QUEUE_TIMEOUT = 3,
    PLT_NAN_INPUT = 4,
    PLT_CUDA_ERROR = 5,
    PLT_NOT_SUPPORTED = 6,
    PLT_BAD_MATERIAL = 7,
    PLT_TOO_LARGE = 8,
    PLT_BOUNDS_VIOLATION = 9   /* a PLT_BOUNDS_CHECK build found an index outside its buffer */
} plt_status;

/* MaterialType ids, Source/Falcor/Scene/Material/MaterialTypes.slang:36-53 */
typedef enum plt_material_type {
    PLT_MATERIAL_UNKNOWN = 0,
    PLT_MATERIAL_STANDARD = 1,
    PLT_MATERIAL_DIFFUSE = 2,
    PLT_MATERIAL_CONDUCTOR = 3,
    PLT_MATERIAL_DIELECTRIC = 4,
    PLT_MATERIAL_OPAQUE_DIELECTRIC = 5,
    PLT_MATERIAL_THIN_DIELECTRIC = 6,
    PLT_MATERIAL_COATED_CONDUCTOR = 7,
    PLT_MATERIAL_COATED_OPAQUE_DIELECTRIC = 8,
    PLT_MATERIAL_GRATED_CONDUCTOR = 9,
    PLT_MATERIAL_GRATED_OPAQUE_DIELECTRIC = 10,
    PLT_MATERIAL_MULTILAYERED_STACK = 11,
    PLT_MATERIAL_TYPE_COUNT = 12
} plt_material_type;

/* LobeType flags, Source/Falcor/Rendering/Materials/LobeType.slang:36-69 */
typedef enum plt_lobe_type {
    PLT_LOBE_NONE = 0x00,
    PLT_LOBE_DIFFUSE_REFLECTION = 0x01,
    PLT_LOBE_SCATTER_REFLECTION = 0x02,
    PLT_LOBE_DELTA_REFLECTION = 0x04,
    PLT_LOBE_DISPERSIVE_DELTA_REFLECTION = 0x08,
    PLT_LOBE_DIFFUSE_TRANSMISSION = 0x10,
    PLT_LOBE_SCATTER_TRANSMISSION = 0x20,
    PLT_LOBE_DELTA_TRANSMISSION = 0x40,
    PLT_LOBE_DISPERSIVE_DELTA_TRANSMISSION = 0x80,
    PLT_LOBE_DELTA = 0xCC,
    PLT_LOBE_NON_DELTA = 0x33,
    PLT_LOBE_REFLECTION = 0x0F,
    PLT_LOBE_TRANSMISSION = 0xF0,
    PLT_LOBE_ALL = 0xFFFF,
    PLT_LOBE_MATERIAL_SPECIFIC = 0xFF00
} plt_lobe_type;

/* SpectralProfile, BasicMaterialData.slang:43-54 (host C++ layout, 1052 bytes). */
typedef struct plt_spectral_profile {
    float rgb[3];
    float intensity;
    uint32_t bins;
    float min_wavelength;
    float max_wavelength;
    float pdf[PLT_SPECTRAL_MAX_BINS];
    float icdf[PLT_SPECTRAL_MAX_BINS];
} plt_spectral_profile;

/* One material: the MaterialHeader type id plus the BasicMaterialData constant fields in their
 * reference order (BasicMaterialData.slang:63-85).  binary16 fields are raw half bits; integer
 * fields the reference bit-casts through asuint16 (grating type/lobes, layer count in data1[3])
 * are stored as those 16 bits.  Texture handles are not part of the record: textures are
 * unsupported, the constants are used. 80 bytes. */
typedef struct plt_material_record {
    uint32_t type;                      /* plt_material_type */
    uint32_t flags;                     /* PLT_MATERIAL_FLAG_* (MaterialHeader bits the PLT path reads) */
    uint16_t base_color[4];
    uint16_t specular[4];
    uint16_t data1[4];
    uint16_t data2[4];
    uint16_t specular_transmission;
    uint16_t transmission[3];
    uint16_t diffuse_transmission;
    uint16_t volume_scattering[3];
    uint16_t ior;
    uint16_t volume_absorption[3];
    uint16_t volume_anisotropy;
    uint16_t pad0;
    uint32_t emission_spectral_id;
    uint32_t ior_n_spectral_id;
    uint32_t ior_k_spectral_id;
} plt_material_record;

/* A batch of BSDF queries in the local shading frame (N = +z, T = +x, B = +y).
 * Each query mirrors one IMaterialInstance call with ShadingData.V = v:
 *   eval(sd, toEye = w, lobe, beam)       pdf(sd, toLight = w, lambda_hero)
 *   sample(sd, sg, lambda_hero)           lambdaPdf(sd, wo = w, lobe, beam, beam.wavelengths)
 * The incoming beam travels along r = -v (PLTPT forwardUnwindStep: sd.V = -beam.r).  Its
 * tangent t is beam_t, or, when beam_t is NULL, the canonical frame of r used by
 * PLTBeam.constructLocalFrame (PLT.slang:218-223). */
typedef struct plt_bsdf_queries {
    uint32_t n;                         /* number of queries */
    uint32_t hwss;                      /* wavelengths per beam, 1..PLT_MAX_HWSS */
    uint32_t rng_offset;                /* sample(): query i uses UniformSampleGenerator(pixel (j & 0xffff, j >> 16), frame), j = i + rng_offset */
    uint32_t frame;                     /* sample(): sample number of the generator */
    const uint32_t* material;           /* [n] index into the context's material table */
    const float* v;                     /* [3][n] sd.V, unit */
    const float* w;                     /* [3][n] toEye (eval, lambdaPdf) / toLight (pdf), unit */
    const uint32_t* lobe;               /* [n] lobe mask for eval / lambdaPdf; NULL = PLT_LOBE_ALL */
    const float* wavelengths;           /* [hwss][n] nm; plane 0 is the hero wavelength */
    const float* stokes;                /* [4*hwss][n] plane (c*hwss + j) = Stokes component c of wavelength j */
    const float* coherence;             /* [4][n] diffusivity D.x, D.y, D.z and distance r_m (m) */
    const float* beam_t;                /* [3][n] beam tangent, or NULL */
} plt_bsdf_queries;

/* Outputs; each pointer may be NULL, and only the requested outputs are written. */
typedef struct plt_bsdf_results {
    float* stokes;                      /* [4*hwss][n] beam Stokes after eval */
    float* coherence;                   /* [4][n] beam coherence after eval (D, r_m) */
    float* beam_t;                      /* [3][n] beam tangent after eval (beam r after eval = w) */
    float* pdf;                         /* [n] pdf(sd, toLight = w, hero wavelength) */
    float* lambda_pdf;                  /* [hwss][n] lambdaPdf(sd, w, lobe, beam, wavelengths) */
    float* sample_wo;                   /* [3][n] sampled direction */
    float* sample_pdf;                  /* [n] */
    float* sample_weight;               /* [n] */
    uint32_t* sample_lobe;              /* [n] sampled LobeType (grating lobe code in bits 8-15) */
    uint32_t* sample_valid;             /* [n] 1 if sample() returned true */
} plt_bsdf_results;

/* Operations of plt_bsdf_batch; OR them together.  Outputs of an unrequested op are untouched. */
#define PLT_OP_EVAL 0x1u
#define PLT_OP_PDF 0x2u
#define PLT_OP_SAMPLE 0x4u
#define PLT_OP_LAMBDA_PDF 0x8u

/* A batch of rays (device SoA planes).  Hits are accepted for tmin <= t <= tmax; triangles are
 * two-sided (the reference traces with RAY_FLAG_NONE / ACCEPT_FIRST_HIT_AND_END_SEARCH, no
 * culling: RenderPasses/PLTPT/ShadowRays.slangh:65-135, pltpt_sample.rt.slang:168-183). */
typedef struct plt_rays {
    uint32_t n;
    const float* origin;                /* [3][n] */
    const float* dir;                   /* [3][n], need not be normalised */
    const float* tmin;                  /* [n], or NULL for 0 */
    const float* tmax;                  /* [n], or NULL for FLT_MAX */
    uint64_t* stats;                    /* [2] device counters (+= BVH node visits, triangle tests), or NULL */
} plt_rays;

/* Closest-hit results: the triangle index (input order of plt_set_scene) with the lowest distance,
 * ties broken by the lowest index; 0xFFFFFFFF on a miss. */
typedef struct plt_hits {
    uint32_t* prim;                     /* [n] */
    float* t;                           /* [n] distance (-1 on a miss), or NULL */
    float* bary;                        /* [2][n] barycentrics of vertices 1 and 2, or NULL */
} plt_hits;

/* PLTPT pass options (RenderPasses/PLTPT/PLTPT.h:74-108, parsed at PLTPT.cpp:147-175). */
typedef struct plt_options {
    uint32_t max_bounces;               /* maxBounces, default 32 */
    uint32_t tile_size;                 /* tileSize, default 512 */
    uint32_t hwss;                      /* HWSS, default 4 */
    uint32_t hwss_do_mis;               /* HWSSDoMIS, default 1 */
    float sourcing_area_from_emissive_geometry; /* mm^2, default 1 */
    float sourcing_max_beam_omega;      /* default 0.025 */
    uint32_t use_direct_light;          /* default 1 */
    uint32_t use_env_light;             /* default 1 */
    uint32_t use_emissive_lights;       /* default 1 */
    uint32_t use_analytic_lights;       /* default 1 */
    uint32_t do_nee;                    /* default 1 */
    uint32_t do_mis;                    /* default 1 */
    uint32_t do_russian_roulette;       /* default 1 */
    uint32_t nee_use_per_tile_sg;       /* default 0 */
    uint32_t do_importance_sample_emitters; /* default 1 */
    uint32_t do_mnee;                   /* default 1 */
    uint32_t mnee_max_occluders;        /* default 2 */
    uint32_t mnee_max_iterations;       /* default 60 */
    float mnee_solver_threshold;        /* default 5e-5 */
    uint32_t flags;                     /* PLT_OPTION_* */
    /* Learned MIS proposal (no counterpart in the reference): when non-zero, plt_render samples
     * every proposal vertex (a material with non-delta lobes other than PLTDiffuse, hit from the
     * front) with the context's proposal network with probability learned_proposal_prob and with
     * the analytic sampler otherwise (one-sample MIS; the exact BSDF is always evaluated).
     * Requires plt_proposal_init or plt_proposal_set_params first. */
    uint32_t learned_proposal;          /* default 0 */
    float learned_proposal_prob;        /* in (0, 1), default 0.5 */
    uint32_t emissive_sampler;          /* emissiveSampler: 0 Uniform, 2 Power (EmissiveLightSamplerType), default 2 */
    uint32_t debug_view;                /* debugView: a PLT_DEBUG_VIEW_* value (DebugViewType.slangh), default 0 (none) */
    float debug_view_intensity;         /* debugViewIntensity: lerp(colour, debug colour, intensity), default 1 */
    uint32_t alpha_masking;             /* alphaMasking: hits on alpha-0 materials pass through, default 1 */
    uint32_t sample_generator;          /* sampleGenerator: PLT_SAMPLE_GENERATOR_*, default 1 (uniform) */
} plt_options;

/* debugView values (RenderPasses/PLTPT/DebugViewType.slangh).  The debug colour of a pixel is the
 * mean of the values each view writes along its path (pltpt_debug.slangh); colour-coded scalars
 * use the magma (path length, spectral samples, coherence area) or inferno (coherence anisotropy,
 * MNEE iterations) colour maps (ColourCoding.slang). */
#define PLT_DEBUG_VIEW_NONE 0u
#define PLT_DEBUG_VIEW_NANS 1u
#define PLT_DEBUG_VIEW_INFS 2u
#define PLT_DEBUG_VIEW_PATH_LENGTH 3u
#define PLT_DEBUG_VIEW_HWSS_COMPS 4u
#define PLT_DEBUG_VIEW_NORMALS 5u
#define PLT_DEBUG_VIEW_ALBEDO 6u
#define PLT_DEBUG_VIEW_ROUGHNESS 7u
#define PLT_DEBUG_VIEW_UVS 8u
#define PLT_DEBUG_VIEW_COHERENCE_AREA 9u
#define PLT_DEBUG_VIEW_COHERENCE_ANISOTROPY 10u
#define PLT_DEBUG_VIEW_POLARIZATION 11u
#define PLT_DEBUG_VIEW_MNEE_ITERATIONS 12u
#define PLT_DEBUG_VIEW_MNEE_BOUNCES 13u

/* sampleGenerator values (Utils/Sampling/SampleGeneratorType.slangh): TinyUniformSampleGenerator
 * (a TEA-seeded 32-bit LCG) and UniformSampleGenerator (SplitMix64-seeded xoshiro128**). */
#define PLT_SAMPLE_GENERATOR_TINY_UNIFORM 0u
#define PLT_SAMPLE_GENERATOR_UNIFORM 1u

#define PLT_OPTION_FP64_MULTILAYER 0x1u /* multilayer recursion in FP64 instead of the reference FP32 */
/* complex-IOR conductor Fresnel (Fresnel.slang:60-73) in FP64 where cos(theta_i) < 0.1 (grazing
 * incidence), for every conductor surface: conductor, coated conductor and grated conductor */
#define PLT_OPTION_FP64_CONDUCTOR_GRAZING 0x10u
#define PLT_OPTION_NO_GRAPH 0x2u        /* plt_render*: launch each frame directly instead of replaying its recorded CUDA graph */
/* Failure injection for tests of the device-side error paths (no counterpart in the reference).
 * Neither faults, traps or hangs the GPU: each makes a bounded condition trip and the kernels
 * report it in the status word that plt_check_status returns (PLT_QUEUE_TIMEOUT), leaving the
 * context usable.  FAULT_COPY_WAIT: the BSDF shade kernel's wait for its spectral-table copy gives
 * up at once (the CTAs then let the copy land and return without shading).  FAULT_SHORT_STACK:
 * plt_trace_* traverse with a 2-entry stack, so deep rays overflow it. */
#define PLT_OPTION_FAULT_COPY_WAIT 0x4u
#define PLT_OPTION_FAULT_SHORT_STACK 0x8u
/* plt_render*: replay every beam through its path inside the solve kernel instead of deferring the
 * replays to the material-sorted replay wavefront (same results up to float summation order) */
#define PLT_OPTION_INLINE_REPLAY 0x20u

typedef struct plt_context plt_context;

/* Library identity. */
uint32_t plt_abi_version(void);
const char* plt_status_string(plt_status status);

/* Fills the PLTPT defaults (PLTPT.h:74-108). Host pointer. */
plt_status plt_options_default(plt_options* out);

/* Replaces PLTPT::create(device, Dictionary) (PLTPT.cpp:147-204): a context on the current
 * CUDA device.  options may be NULL (defaults).  Host pointers. */
plt_status plt_create(const plt_options* options, plt_context** out);
plt_status plt_destroy(plt_context* ctx);
int plt_last_cuda_error(const plt_context* ctx);

/* Replaces the scene's spectral-profile buffer upload (Scene.cpp:765-792): host array. */
plt_status plt_set_spectral_profiles(plt_context* ctx, const plt_spectral_profile* profiles, uint32_t count);

/* Replaces MaterialSystem upload of BasicMaterialData + setupMaterialInstance decoding
 * (MaterialFactory.slang:79-130, PLT*Material.slang): host array.  Records are validated
 * (type id, spectral ids in range) and decoded once into the device material table. */
plt_status plt_set_materials(plt_context* ctx, const plt_material_record* materials, uint32_t count);

/* Builds a SpectralProfile from piecewise-linear samples (.spd data), restating
 * PiecewiseLinearSpectrum::eval (Utils/Color/Spectrum.h:88-107), SampledSpectrum
 * (Utils/Color/SampledSpectrum.h:64-73,308-317) and genSpectralProfile
 * (SceneBuilder.cpp:911-960).  Host pointers. */
plt_status plt_spectral_profile_from_samples(const float* wavelengths_nm, const float* values,
                                             uint32_t count, float scale, int compute_icdf,
                                             plt_spectral_profile* out);

/* Reads a .spd spectral table (wavelength nm, value per line; '#' and blank lines skipped; reading
 * stops at the first other line, PiecewiseLinearSpectrum::fromFile, Utils/Color/Spectrum.cpp:89-111)
 * and builds its SpectralProfile as plt_spectral_profile_from_samples.  Host path and pointer. */
plt_status plt_spectral_profile_from_spd(const char* path, float scale, int compute_icdf, plt_spectral_profile* out);

/* The reference's spectral-table lookups by name (tables_dir = a directory laid out as the
 * reference's Source/Tables: ior/<name>.eta.spd + ior/<name>.k.spd, emission/<name>.spd).
 * Replaces SceneBuilder::addSpectralProfileFromMaterial ("none" = constant n 1, k 0; no inverse
 * CDF) and SceneBuilder::addSpectralProfileForEmitterType (scaled, with inverse CDF)
 * (Scene/SceneBuilder.cpp:967-993).  PLT_INVALID_ARG when a table is missing.  Host pointers. */
plt_status plt_spectral_profiles_from_material(const char* tables_dir, const char* name, plt_spectral_profile* eta,
                                               plt_spectral_profile* k);
plt_status plt_spectral_profile_for_emitter_type(const char* tables_dir, const char* name, float scale, plt_spectral_profile* out);

/* Writes an RGBA image ([height][width][4] floats, host) as an uncompressed scanline OpenEXR file,
 * HALF channels when half != 0, else FLOAT (the reference's pass graph ends in an accumulated EXR
 * capture, scripts/PLTPathTracer.py:19-27). */
plt_status plt_write_exr(const char* path, const float* rgba, uint32_t width, uint32_t height, int half);

/* plt_bsdf_batch with HOST queries and results (same structures, host pointers; pinned memory
 * gives full copy bandwidth).  The batch is pipelined in chunks of 2^21 queries: input copies,
 * kernels and output copies of different chunks (and of consecutive calls) overlap on the
 * library's two copy streams and compute stream; the results equal one plt_bsdf_batch over the
 * whole batch.  Asynchronous and ordered on `stream`: no input is read before the work queued on
 * `stream` ahead of the call has completed (so inputs that earlier work on `stream` writes are
 * read complete), and the results are on the host once `stream` has completed.  The pipeline
 * sorts through its own scratch, so it shares no scratch with plt_bsdf_batch.  Holds four staging
 * slots of device memory until plt_destroy, each sized for the largest chunk seen (132 bytes per
 * query of a chunk at HWSS 1 with every op: about 277 MB for 2^21 queries). */
plt_status plt_bsdf_batch_host(plt_context* ctx, const plt_bsdf_queries* queries,
                               const plt_bsdf_results* results, uint32_t ops, void* stream);

/* Batched IMaterialInstance calls (see plt_bsdf_queries).  ops = PLT_OP_* mask.  One fused
 * launch serves every requested op; queries may mix materials in any order.  Every launching entry
 * point (batches, traversal, renders) must be called with the context's device current, else it
 * returns PLT_INVALID_ARG.  Calls on one context share its sort scratch: queue them on one stream
 * (or order them with events). */
plt_status plt_bsdf_batch(plt_context* ctx, const plt_bsdf_queries* queries,
                          const plt_bsdf_results* results, uint32_t ops, void* stream);

/* Replaces the scene's DXR acceleration-structure build (Scene/Scene.cpp:3092-3764): a binned-SAH
 * BVH over the triangles is built on the host and uploaded.  Host arrays: vertices [n_vertices][3],
 * indices [n_triangles][3], material [n_triangles] (material index per triangle, or NULL for 0). */
plt_status plt_set_scene(plt_context* ctx, const float* vertices, uint32_t n_vertices, const uint32_t* indices,
                         uint32_t n_triangles, const uint32_t* material);

/* Closest hit per ray (replaces TraceRay with a closest-hit shader), and occlusion per ray
 * (replaces visibility rays with ACCEPT_FIRST_HIT_AND_END_SEARCH): occluded[i] = 1 if any triangle
 * is hit with tmin <= t <= tmax.  Device pointers, asynchronous on `stream`. */
plt_status plt_trace_closest(plt_context* ctx, const plt_rays* rays, const plt_hits* hits, void* stream);
plt_status plt_trace_any(plt_context* ctx, const plt_rays* rays, uint32_t* occluded, void* stream);

/* BVH statistics of the current scene (host pointer, 4 values: nodes, leaves, max depth, triangles). */
plt_status plt_scene_stats(const plt_context* ctx, uint32_t* out4);

/* Per-vertex shading attributes of the current scene, StaticVertexData.normal / .tangent
 * (Scene/SceneTypes.slang) in world space (the scene has identity instance transforms): normals
 * [n_vertices][3] (required before plt_render), tangents [n_vertices][4] (xyz + handedness sign w;
 * NULL = no tangent space, the shading frame is then built with perp_stark as in
 * ShadingUtils.slang:126-153), tri_instance [n_triangles] the geometry instance (mesh) of each
 * triangle, which manifold walks re-project onto (Manifolds.slangh:246-248; NULL = one instance).
 * Host arrays, copied.  Also builds the emissive-triangle list and the power sampler's alias table
 * from the materials set with plt_set_materials, so call it after both plt_set_scene and
 * plt_set_materials (and again when either changes). */
plt_status plt_set_scene_shading(plt_context* ctx, const float* normals, const float* tangents, uint32_t n_vertices,
                                 const uint32_t* tri_instance);

/* Material double-sidedness, MaterialHeader::isDoubleSided (Scene/Material/MaterialData.slang:126-130),
 * carried in plt_material_record.flags; transmissive records are double-sided regardless
 * (BasicMaterial::adjustDoubleSidedFlag, BasicMaterial.cpp:719-731). */
#define PLT_MATERIAL_FLAG_DOUBLE_SIDED 0x1u

/* Pinhole camera: the CameraData fields computeRayPinhole (Scene/Camera/Camera.slang:46-78) and
 * the solve pass's polarizer (pltpt_solve.rt.slang:110-124) read. */
typedef struct plt_camera {
    float pos[3];                       /* posW */
    float u[3], v[3], w[3];             /* cameraU, cameraV, cameraW as Falcor stores them (unnormalised) */
    float jitter_x, jitter_y;           /* jitterX, jitterY */
    float polarizer;                    /* polarizer intensity, 0 = none */
    float polarizer_theta;              /* polarizer angle (rad) */
} plt_camera;

/* Renders `frame_count` frames (gFrameCount = frame_begin + f) of the PLTPT pass: per frame a sample
 * pass (backward path construction into the bounce buffer) and a solve pass (NEE, emissive hits,
 * forward beam replay, spectral MIS, measurement), as PLTPT::execute (PLTPT.cpp:357-499) does per
 * tile.  out_rgba [height][width][4] (device) receives the mean of the frames' gOutputColor
 * (AccumulatePass, scripts/PLTPathTracer.py:19).  Options come from plt_create; hwss 1-4. */
plt_status plt_render(plt_context* ctx, const plt_camera* camera, uint32_t width, uint32_t height, uint32_t frame_begin,
                      uint32_t frame_count, float* out_rgba, void* stream);

/* Environment light: replaces Scene::setEnvMap / EnvMap (Scene/Lights/EnvMap.cpp:60-126,
 * EnvMap.slang) and EnvMapSampler (Rendering/Lights/EnvMapSampler.cpp:85-120,
 * EnvMapSampler.slang).  pixels: host [height][width][channels] linear RGB(A) lat-long map (the
 * map is centred on -z, world_to_latlong_map), values finite and >= 0; intensity >= 0; tint (3, or
 * NULL = white) and rotation_deg (Euler XYZ degrees, or NULL = none) as EnvMap's setTint /
 * setRotation.  Builds the sampler's 512 x 512 importance map on the device.  With options
 * use_env_light (default 1), plt_render and plt_render_scenes then sample the map in NEE
 * (light-type selection between the map and emissive geometry, LightSampling.slangh:40-206) and
 * add it on escaped paths (onMiss, pltpt_solve.rt.slang:374-395), for every scene of the context. */
plt_status plt_set_env_map(plt_context* ctx, const float* pixels, uint32_t width, uint32_t height, uint32_t channels,
                           float intensity, const float* tint, const float* rotation_deg);
plt_status plt_clear_env_map(plt_context* ctx);
/* The sampler on given inputs (device arrays; for tests): for each i, sample(u[2i], u[2i+1]) and
 * the map's eval / evalPdf at the sampled direction and at dirs[3i..3i+2] (dirs may be NULL).
 * out[12i..12i+11] = sampled direction (3), its pdf, eval rgb (3), evalPdf, eval rgb of dirs[i]
 * (3), evalPdf of dirs[i].  PLT_INVALID_ARG without an environment map. */
plt_status plt_env_map_query(plt_context* ctx, const float* u, const float* dirs, uint32_t n, float* out, void* stream);

/* Analytic lights: LightData (Scene/Lights/LightData.slang:36-67) as the scene's light classes fill
 * it (Scene/Lights/Light.cpp), for NEE's third light type (generateAnalyticLightSample,
 * RenderPasses/PLTPT/LightSampling.slangh:128-164, sampleLight, Rendering/Lights/LightHelpers.slang).
 * With options use_analytic_lights (default 1) and at least one light, light-type selection picks
 * among the environment map, emissive geometry and these lights; a light is chosen uniformly.  As
 * in the reference, point (spot) and directional lights have a zero pdf and their samples are
 * rejected, analytic lights are never MIS-weighted and never hit by rays, and an area light's beam
 * is sourced at pos (LightData.posW, left at the origin by the area-light classes).  The lights
 * apply to every scene of the context.  Host array, copied. */
typedef enum plt_light_type {
    PLT_LIGHT_POINT = 0,
    PLT_LIGHT_DIRECTIONAL = 1,
    PLT_LIGHT_DISTANT = 2,
    PLT_LIGHT_RECT = 3,
    PLT_LIGHT_DISC = 4,
    PLT_LIGHT_SPHERE = 5
} plt_light_type;
typedef struct plt_analytic_light {
    uint32_t type;                      /* plt_light_type */
    uint32_t intensity_spectral_id;     /* spectral profile of the intensity */
    float pos[3];                       /* posW */
    float dir[3];                       /* dirW (normalised) */
    float opening_angle;                /* spot: half-angle, pi = full sphere */
    float cos_opening_angle;
    float penumbra_angle;
    float cos_subtended_angle;          /* distant light */
    float surface_area;                 /* area lights, as the light class's update() computes it */
    float transform[12];                /* transMat rows 0-2 (row-major 3x4): area lights, distant light frame */
} plt_analytic_light;
plt_status plt_set_analytic_lights(plt_context* ctx, const plt_analytic_light* lights, uint32_t count);

/* Scene sets (no counterpart in the reference, whose PLTPT renders the one loaded scene): several
 * independent scenes held by one context share its materials and spectral profiles, and
 * plt_render_scenes renders any number of views of them in one wavefront per frame (all scenes'
 * paths in the same segment, solve and manifold-walk launches; each path traverses its own scene's
 * BVH and samples its own scene's lights).  plt_set_scene replaces the set with one scene;
 * plt_add_scene appends a scene with its shading attributes (same meaning as plt_set_scene +
 * plt_set_scene_shading; host arrays, copied) and returns its index; plt_clear_scenes empties the
 * set.  plt_set_scene_shading applies to the most recently set or added scene.  The trace entry
 * points and plt_render use scene 0. */
#define PLT_MAX_SCENES 4096u
typedef struct plt_scene_desc {
    const float* positions;             /* [n_vertices][3] */
    uint32_t n_vertices;
    const uint32_t* indices;            /* [n_triangles][3] */
    uint32_t n_triangles;
    const uint32_t* tri_material;       /* [n_triangles] or NULL (material 0) */
    const float* normals;               /* [n_vertices][3] */
    const float* tangents;              /* [n_vertices][4] or NULL */
    const uint32_t* tri_instance;       /* [n_triangles] or NULL */
} plt_scene_desc;
plt_status plt_add_scene(plt_context* ctx, const plt_scene_desc* desc, uint32_t* out_scene);
plt_status plt_clear_scenes(plt_context* ctx);

/* One view of a scene-set render: the scene index, camera, image size and the device output image
 * [height][width][4] (16-byte aligned). */
typedef struct plt_render_view {
    uint32_t scene;
    uint32_t width, height;
    uint32_t pad;
    plt_camera camera;
    float* out_rgba;
} plt_render_view;
/* Renders frame_count frames of every view (the same frame indices for all views; each view's
 * pixels seed the generator exactly as a plt_render of that view alone, so the results equal
 * n separate plt_render calls).  At most 2^26 pixels over all views. */
plt_status plt_render_scenes(plt_context* ctx, const plt_render_view* views, uint32_t n_views, uint32_t frame_begin, uint32_t frame_count,
                             void* stream);

/* Launch shape of the render pass (no counterpart in the reference): the frame's paths of all views
 * are processed in waves of at most wave_paths paths (0 = one wave; smaller waves bound the path
 * state and bounce records and keep them cache-resident between the sample and solve passes), and
 * the segment, solve and manifold-walk kernels run with the given blocks of 128 per SM (0 = the
 * occupancy limit).  The solve pass takes a large wave's paths sorted by length, longest first, so a
 * warp's paths need similar work (path_order selects: see the field).  Results do not depend on the shape.  plt_render_tune times a coordinate
 * search over the shape on the caller's views (frames frame, frame + 1, ...; the views' outputs are
 * overwritten), keeps the fastest for later renders and returns it with its time per frame. */
typedef struct plt_launch_shape {
    uint32_t wave_paths;
    uint32_t segment_blocks_per_sm, solve_blocks_per_sm, walk_blocks_per_sm;
    uint32_t path_order;                /* 0: longest first for waves of >= 2^18 paths; 1: path order; 2: always longest first */
} plt_launch_shape;
plt_status plt_set_launch_shape(plt_context* ctx, const plt_launch_shape* shape);   /* NULL = defaults */
plt_status plt_get_launch_shape(const plt_context* ctx, plt_launch_shape* shape);
plt_status plt_render_tune(plt_context* ctx, const plt_render_view* views, uint32_t n_views, uint32_t frame, uint32_t frames,
                           plt_launch_shape* best, float* best_ms, void* stream);

/* Path statistics of the last plt_render frame (host pointer, 4 values: paths, bounces recorded,
 * shadow rays traced, forward-unwind BSDF evaluations). */
plt_status plt_render_stats(plt_context* ctx, uint64_t* out4);

/* Counters of the last frame of the last render (host pointer, the first n of: paths of all
 * views, bounces recorded, shadow rays traced, forward-unwind BSDF evaluations, algorithmic
 * traversal bytes = 64 per BVH node visited + 48 per triangle tested over all rays). */
plt_status plt_render_counters(plt_context* ctx, uint64_t* out, uint32_t n);

/* The bounce buffer of the last plt_render frame (Path.slang BounceData per path and bounce), for
 * inspection: host arrays [width*height][max_bounces+1] of the hit triangle (0xFFFFFFFF when the
 * record is absent or a miss), the sampled lobe and the RayFlags word; any may be NULL.
 * Synchronises the device. */
plt_status plt_render_bounces(plt_context* ctx, uint32_t* prim, uint32_t* lobe, uint32_t* flags);

/* Synchronises `stream`, then reports and clears the context's device status word, which every
 * launch since the previous check ORs into: PLT_BOUNDS_VIOLATION (a library built with
 * -DPLT_BOUNDS_CHECK=1 found an index outside its buffer; see plt_last_bounds_violation),
 * PLT_BAD_MATERIAL (a material index out of range or of an unknown type; those queries return
 * zeros), PLT_NAN_INPUT (a non-finite direction or wavelength), PLT_QUEUE_TIMEOUT (a bounded device
 * wait gave up or a traversal stack overflowed).  Mirrors the reference's logError/throw reporting
 * (PLTPT.cpp:173,409), which has no device-side status. */
plt_status plt_check_status(plt_context* ctx, void* stream);

/* The first bounds violation of the launches that the last plt_check_status returning
 * PLT_BOUNDS_VIOLATION covered (host pointer, 3 values): the site (1 queue entry, 2 path id, 3
 * bounce record, 4 triangle, 5 material, 6 deferred task, 7 image accumulator, 8 batch query, 9
 * sort permutation), the index and the buffer's bound; zeros when there was none.  Only a library
 * built with -DPLT_BOUNDS_CHECK=1 checks indices (the default build does not). */
plt_status plt_last_bounds_violation(const plt_context* ctx, uint32_t* out3);

/* Learned MIS proposal (no counterpart in the reference, whose PLTPT samples only the analytic
 * BSDF samplers).  A conditional MLP 16 -> 64 -> 64 -> 64 -> 32 with SiLU maps the features of a
 * query -- wi (3, shading frame, z >= 0), (wavelength - 550) / 170, roughness, grating pitch / 5 um,
 * material class one-hot (8), two zero pads -- to 8 x (logit, mu_x, mu_y, log sigma): a mixture of
 * isotropic Gaussians over the primary sample (u0, u1) in [0,1)^2 that the material's surface model
 * (Gaussian or fractal) maps to a non-delta direction.  BF16 weights and activations, FP32
 * accumulation on the tensor cores.  The render pass uses it as an extra one-sample MIS technique
 * in primary sample space (plt_options.learned_proposal): the path weight is divided by the
 * primary sample's mixture density, so the estimate has the analytic tracer's expectation.  Parameters
 * are FP32 on the host side of these calls, in the order W1 [64][16], W2 [64][64], W3 [64][64],
 * W4 [32][64], b1, b2, b3, b4.  Training samples come from the exact non-delta samplers of the
 * context's materials (set them first). */
#define PLT_PROPOSAL_PARAMS 11488u
#define PLT_PROPOSAL_FEATURES 16u
#define PLT_PROPOSAL_OUTPUTS 32u
plt_status plt_proposal_init(plt_context* ctx, uint64_t seed);
plt_status plt_proposal_set_params(plt_context* ctx, const float* params);   /* host [PLT_PROPOSAL_PARAMS] */
plt_status plt_proposal_get_params(plt_context* ctx, float* params);         /* host [PLT_PROPOSAL_PARAMS] */
/* n training samples (device): x [n][16] bf16 bits, target [n][2] (the uniform primary sample the
 * surface model turned into a non-delta direction), weight [n] (that direction's BSDF value over the
 * sampler's pdf for an unpolarised beam, clamped to 4; 0 = no sample). */
plt_status plt_proposal_generate(plt_context* ctx, uint32_t n, uint32_t seed, uint16_t* x, float* target, float* weight, void* stream);
/* grad [PLT_PROPOSAL_PARAMS] (device, overwritten) and loss [1] (device) of the mean weighted
 * negative log-likelihood of the batch under the current parameters. */
plt_status plt_proposal_gradient(plt_context* ctx, uint32_t n, const uint16_t* x, const float* target, const float* weight, float* grad,
                                 float* loss, void* stream);
/* out [n][32] (device, fp32): the network outputs for feature rows x. */
plt_status plt_proposal_forward(plt_context* ctx, uint32_t n, const uint16_t* x, float* out, void* stream);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) with a device gradient. */
plt_status plt_proposal_adam_step(plt_context* ctx, const float* grad, float lr, void* stream);
/* steps x (generate batch, gradient, Adam); loss_history (host [steps]) may be NULL.  Initialises
 * the parameters from `seed` when none are set. */
plt_status plt_proposal_train(plt_context* ctx, uint32_t steps, uint32_t batch, float lr, uint32_t seed, float* loss_history, void* stream);

/* Per-kernel timing of plt_bsdf_batch (a profiling aid; no counterpart in the reference, whose
 * shaders are timed only as a whole render pass).  Each later plt_bsdf_batch
 * on this context records the given cudaEvent_t handles (any may be NULL) on its stream: before the
 * classify kernel, between classify and shade, and after the shade kernel (a batch of at most 65,536
 * queries is not classified: the first two events are recorded back to back).  NULLs switch it off. */
plt_status plt_set_timing_events(plt_context* ctx, void* before_classify, void* before_shade, void* after_shade);

/* Largest batch plt_bsdf_batch_noalloc accepts. */
#define PLT_NOALLOC_MAX_QUERIES (1u << 20)

/* plt_bsdf_batch for callers that must not allocate device memory -- for example a renderer's
 * per-frame loop running under a fixed memory budget, or a host application that owns all device
 * allocations and forbids libraries to call cudaMalloc (which can synchronise the device and fail
 * under memory pressure).  It has no counterpart in the reference, whose shaders run inside the
 * graphics API's own memory management.  Same arguments and results as plt_bsdf_batch; the
 * batch's sorting scratch lives in a fixed device array of the library (about 2 MB per GPU, held
 * until exit) instead of context memory, so the call itself allocates nothing.
 * Limits: queries->n <= PLT_NOALLOC_MAX_QUERIES, else PLT_TOO_LARGE (nothing launched).  The
 * first call on each device resolves the array's device address (set-up); make that first call
 * before starting any stream capture.  Like plt_bsdf_batch it runs only with the context's device
 * current (PLT_INVALID_ARG otherwise).  Calls share the array: calls that overlap on the GPU race,
 * so serialise them on one stream.  Not usable after a cudaDeviceReset in the same process. */
plt_status plt_bsdf_batch_noalloc(plt_context* ctx, const plt_bsdf_queries* queries,
                                  const plt_bsdf_results* results, uint32_t ops, void* stream);

/* Single-op conveniences over plt_bsdf_batch. */
plt_status plt_bsdf_eval(plt_context* ctx, const plt_bsdf_queries* q, const plt_bsdf_results* r, void* stream);
plt_status plt_bsdf_pdf(plt_context* ctx, const plt_bsdf_queries* q, const plt_bsdf_results* r, void* stream);
plt_status plt_bsdf_sample(plt_context* ctx, const plt_bsdf_queries* q, const plt_bsdf_results* r, void* stream);
plt_status plt_bsdf_lambda_pdf(plt_context* ctx, const plt_bsdf_queries* q, const plt_bsdf_results* r, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PLT_GB300_H */
