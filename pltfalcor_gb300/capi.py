"""ctypes mirror of include/plt_gb300.h and the loader of libplt_gb300.so.

The library is built in-tree (pltfalcor_gb300/_build/libplt_gb300.so) by pltfalcor_gb300.build;
loading fails loudly when it is missing: there is no CPU fallback for the GPU path.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libplt_gb300.so")

PLT_OK, PLT_INVALID_ARG, PLT_OOM, PLT_QUEUE_TIMEOUT, PLT_NAN_INPUT, PLT_CUDA_ERROR, PLT_NOT_SUPPORTED, PLT_BAD_MATERIAL = range(8)
STATUS_NAMES = {0: "PLT_OK", 1: "PLT_INVALID_ARG", 2: "PLT_OOM", 3: "PLT_QUEUE_TIMEOUT", 4: "PLT_NAN_INPUT",
                5: "PLT_CUDA_ERROR", 6: "PLT_NOT_SUPPORTED", 7: "PLT_BAD_MATERIAL"}

OP_EVAL, OP_PDF, OP_SAMPLE, OP_LAMBDA_PDF = 0x1, 0x2, 0x4, 0x8
OP_ALL = 0xF
MAX_HWSS = 8
NO_SPECTRAL_PROFILE = 0xFFFFFFFF
OPTION_FP64_MULTILAYER = 0x1
OPTION_FP64_CONDUCTOR_GRAZING = 0x10
OPTION_FAULT_COPY_WAIT = 0x4
OPTION_FAULT_SHORT_STACK = 0x8
OPTION_INLINE_REPLAY = 0x20


class SpectralProfile(C.Structure):
    _fields_ = [("rgb", C.c_float * 3), ("intensity", C.c_float), ("bins", C.c_uint32),
                ("min_wavelength", C.c_float), ("max_wavelength", C.c_float),
                ("pdf", C.c_float * 128), ("icdf", C.c_float * 128)]


class MaterialRecord(C.Structure):
    _fields_ = [("type", C.c_uint32), ("flags", C.c_uint32),
                ("base_color", C.c_uint16 * 4), ("specular", C.c_uint16 * 4),
                ("data1", C.c_uint16 * 4), ("data2", C.c_uint16 * 4),
                ("specular_transmission", C.c_uint16), ("transmission", C.c_uint16 * 3),
                ("diffuse_transmission", C.c_uint16), ("volume_scattering", C.c_uint16 * 3),
                ("ior", C.c_uint16), ("volume_absorption", C.c_uint16 * 3), ("volume_anisotropy", C.c_uint16),
                ("pad0", C.c_uint16), ("emission_spectral_id", C.c_uint32), ("ior_n_spectral_id", C.c_uint32),
                ("ior_k_spectral_id", C.c_uint32)]


class BsdfQueries(C.Structure):
    _fields_ = [("n", C.c_uint32), ("hwss", C.c_uint32), ("rng_offset", C.c_uint32), ("frame", C.c_uint32),
                ("material", C.c_void_p), ("v", C.c_void_p), ("w", C.c_void_p), ("lobe", C.c_void_p),
                ("wavelengths", C.c_void_p), ("stokes", C.c_void_p), ("coherence", C.c_void_p), ("beam_t", C.c_void_p)]


class BsdfResults(C.Structure):
    _fields_ = [("stokes", C.c_void_p), ("coherence", C.c_void_p), ("beam_t", C.c_void_p), ("pdf", C.c_void_p),
                ("lambda_pdf", C.c_void_p), ("sample_wo", C.c_void_p), ("sample_pdf", C.c_void_p),
                ("sample_weight", C.c_void_p), ("sample_lobe", C.c_void_p), ("sample_valid", C.c_void_p)]


class Rays(C.Structure):
    _fields_ = [("n", C.c_uint32), ("origin", C.c_void_p), ("dir", C.c_void_p), ("tmin", C.c_void_p), ("tmax", C.c_void_p),
                ("stats", C.c_void_p)]


class Hits(C.Structure):
    _fields_ = [("prim", C.c_void_p), ("t", C.c_void_p), ("bary", C.c_void_p)]


class Options(C.Structure):
    _fields_ = [("max_bounces", C.c_uint32), ("tile_size", C.c_uint32), ("hwss", C.c_uint32),
                ("hwss_do_mis", C.c_uint32), ("sourcing_area_from_emissive_geometry", C.c_float),
                ("sourcing_max_beam_omega", C.c_float), ("use_direct_light", C.c_uint32),
                ("use_env_light", C.c_uint32), ("use_emissive_lights", C.c_uint32),
                ("use_analytic_lights", C.c_uint32), ("do_nee", C.c_uint32), ("do_mis", C.c_uint32),
                ("do_russian_roulette", C.c_uint32), ("nee_use_per_tile_sg", C.c_uint32),
                ("do_importance_sample_emitters", C.c_uint32), ("do_mnee", C.c_uint32),
                ("mnee_max_occluders", C.c_uint32), ("mnee_max_iterations", C.c_uint32),
                ("mnee_solver_threshold", C.c_float), ("flags", C.c_uint32),
                ("learned_proposal", C.c_uint32), ("learned_proposal_prob", C.c_float), ("emissive_sampler", C.c_uint32),
                ("debug_view", C.c_uint32), ("debug_view_intensity", C.c_float), ("alpha_masking", C.c_uint32),
                ("sample_generator", C.c_uint32)]

DEBUG_VIEW_NONE, DEBUG_VIEW_NANS, DEBUG_VIEW_INFS, DEBUG_VIEW_PATH_LENGTH, DEBUG_VIEW_HWSS_COMPS, DEBUG_VIEW_NORMALS, \
    DEBUG_VIEW_ALBEDO, DEBUG_VIEW_ROUGHNESS, DEBUG_VIEW_UVS, DEBUG_VIEW_COHERENCE_AREA, DEBUG_VIEW_COHERENCE_ANISOTROPY, \
    DEBUG_VIEW_POLARIZATION, DEBUG_VIEW_MNEE_ITERATIONS, DEBUG_VIEW_MNEE_BOUNCES = range(14)
SAMPLE_GENERATOR_TINY_UNIFORM, SAMPLE_GENERATOR_UNIFORM = 0, 1


class Camera(C.Structure):
    _fields_ = [("pos", C.c_float * 3), ("u", C.c_float * 3), ("v", C.c_float * 3), ("w", C.c_float * 3),
                ("jitter_x", C.c_float), ("jitter_y", C.c_float), ("polarizer", C.c_float), ("polarizer_theta", C.c_float)]


class SceneDesc(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("n_vertices", C.c_uint32), ("indices", C.c_void_p), ("n_triangles", C.c_uint32),
                ("tri_material", C.c_void_p), ("normals", C.c_void_p), ("tangents", C.c_void_p), ("tri_instance", C.c_void_p)]


LIGHT_POINT, LIGHT_DIRECTIONAL, LIGHT_DISTANT, LIGHT_RECT, LIGHT_DISC, LIGHT_SPHERE = range(6)


class AnalyticLight(C.Structure):
    _fields_ = [("type", C.c_uint32), ("intensity_spectral_id", C.c_uint32), ("pos", C.c_float * 3), ("dir", C.c_float * 3),
                ("opening_angle", C.c_float), ("cos_opening_angle", C.c_float), ("penumbra_angle", C.c_float),
                ("cos_subtended_angle", C.c_float), ("surface_area", C.c_float), ("transform", C.c_float * 12)]


class RenderView(C.Structure):
    _fields_ = [("scene", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32), ("pad", C.c_uint32),
                ("camera", Camera), ("out_rgba", C.c_void_p)]


class LaunchShape(C.Structure):
    _fields_ = [("wave_paths", C.c_uint32), ("segment_blocks_per_sm", C.c_uint32), ("solve_blocks_per_sm", C.c_uint32),
                ("walk_blocks_per_sm", C.c_uint32), ("path_order", C.c_uint32)]


MATERIAL_FLAG_DOUBLE_SIDED = 0x1
MAX_SCENES = 4096
OPTION_NO_GRAPH = 0x2

assert C.sizeof(SpectralProfile) == 1052
assert C.sizeof(MaterialRecord) == 80

# every symbol include/plt_gb300.h declares
EXPORTED_SYMBOLS = [
    "plt_abi_version", "plt_status_string", "plt_options_default", "plt_create", "plt_destroy",
    "plt_last_cuda_error", "plt_set_spectral_profiles", "plt_set_materials", "plt_spectral_profile_from_samples",
    "plt_bsdf_batch", "plt_check_status", "plt_bsdf_eval", "plt_bsdf_pdf", "plt_bsdf_sample", "plt_bsdf_lambda_pdf",
    "plt_set_scene", "plt_trace_closest", "plt_trace_any", "plt_scene_stats", "plt_bsdf_batch_noalloc",
    "plt_set_timing_events", "plt_set_scene_shading", "plt_render", "plt_render_stats", "plt_render_bounces",
    "plt_proposal_init", "plt_proposal_set_params", "plt_proposal_get_params", "plt_proposal_generate",
    "plt_proposal_gradient", "plt_proposal_forward", "plt_proposal_adam_step", "plt_proposal_train",
    "plt_add_scene", "plt_clear_scenes", "plt_render_scenes", "plt_set_launch_shape", "plt_get_launch_shape", "plt_render_tune",
    "plt_spectral_profile_from_spd", "plt_write_exr", "plt_render_counters",
    "plt_set_env_map", "plt_clear_env_map", "plt_env_map_query",
    "plt_spectral_profiles_from_material", "plt_spectral_profile_for_emitter_type", "plt_set_analytic_lights",
    "plt_bsdf_batch_host", "plt_last_bounds_violation",
]
NOALLOC_MAX_QUERIES = 1 << 20
PROPOSAL_PARAMS = 11488
PLT_TOO_LARGE = 8
STATUS_NAMES[PLT_TOO_LARGE] = "PLT_TOO_LARGE"
PLT_BOUNDS_VIOLATION = 9
STATUS_NAMES[PLT_BOUNDS_VIOLATION] = "PLT_BOUNDS_VIOLATION"

_lib = None


def load_library(path=LIB_PATH):
    """Loads libplt_gb300.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libplt_gb300.so is not built (%s); run __graft_entry__.build()" % path)
    lib = C.CDLL(path)
    vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int
    sig = {
        "plt_abi_version": (u32, []),
        "plt_last_bounds_violation": (i32, [vp, C.POINTER(C.c_uint32)]),
        "plt_status_string": (C.c_char_p, [i32]),
        "plt_options_default": (i32, [C.POINTER(Options)]),
        "plt_create": (i32, [C.POINTER(Options), C.POINTER(vp)]),
        "plt_destroy": (i32, [vp]),
        "plt_last_cuda_error": (i32, [vp]),
        "plt_set_spectral_profiles": (i32, [vp, C.POINTER(SpectralProfile), u32]),
        "plt_set_materials": (i32, [vp, C.POINTER(MaterialRecord), u32]),
        "plt_spectral_profile_from_samples": (i32, [C.POINTER(C.c_float), C.POINTER(C.c_float), u32, C.c_float, i32,
                                                    C.POINTER(SpectralProfile)]),
        "plt_bsdf_batch": (i32, [vp, C.POINTER(BsdfQueries), C.POINTER(BsdfResults), u32, vp]),
        "plt_bsdf_batch_host": (i32, [vp, C.POINTER(BsdfQueries), C.POINTER(BsdfResults), u32, vp]),
        "plt_check_status": (i32, [vp, vp]),
        "plt_bsdf_eval": (i32, [vp, C.POINTER(BsdfQueries), C.POINTER(BsdfResults), vp]),
        "plt_bsdf_pdf": (i32, [vp, C.POINTER(BsdfQueries), C.POINTER(BsdfResults), vp]),
        "plt_bsdf_sample": (i32, [vp, C.POINTER(BsdfQueries), C.POINTER(BsdfResults), vp]),
        "plt_bsdf_lambda_pdf": (i32, [vp, C.POINTER(BsdfQueries), C.POINTER(BsdfResults), vp]),
        "plt_set_scene": (i32, [vp, vp, u32, vp, u32, vp]),
        "plt_trace_closest": (i32, [vp, C.POINTER(Rays), C.POINTER(Hits), vp]),
        "plt_trace_any": (i32, [vp, C.POINTER(Rays), vp, vp]),
        "plt_scene_stats": (i32, [vp, C.POINTER(C.c_uint32)]),
        "plt_bsdf_batch_noalloc": (i32, [vp, C.POINTER(BsdfQueries), C.POINTER(BsdfResults), u32, vp]),
        "plt_set_timing_events": (i32, [vp, vp, vp, vp]),
        "plt_set_scene_shading": (i32, [vp, vp, vp, u32, vp]),
        "plt_render": (i32, [vp, C.POINTER(Camera), u32, u32, u32, u32, vp, vp]),
        "plt_render_stats": (i32, [vp, C.POINTER(C.c_uint64)]),
        "plt_render_bounces": (i32, [vp, vp, vp, vp]),
        "plt_proposal_init": (i32, [vp, C.c_uint64]),
        "plt_proposal_set_params": (i32, [vp, C.POINTER(C.c_float)]),
        "plt_proposal_get_params": (i32, [vp, C.POINTER(C.c_float)]),
        "plt_proposal_generate": (i32, [vp, u32, u32, vp, vp, vp, vp]),
        "plt_proposal_gradient": (i32, [vp, u32, vp, vp, vp, vp, vp, vp]),
        "plt_proposal_forward": (i32, [vp, u32, vp, vp, vp]),
        "plt_proposal_adam_step": (i32, [vp, vp, C.c_float, vp]),
        "plt_proposal_train": (i32, [vp, u32, u32, C.c_float, u32, C.POINTER(C.c_float), vp]),
        "plt_add_scene": (i32, [vp, C.POINTER(SceneDesc), C.POINTER(C.c_uint32)]),
        "plt_clear_scenes": (i32, [vp]),
        "plt_render_scenes": (i32, [vp, C.POINTER(RenderView), u32, u32, u32, vp]),
        "plt_set_launch_shape": (i32, [vp, C.POINTER(LaunchShape)]),
        "plt_get_launch_shape": (i32, [vp, C.POINTER(LaunchShape)]),
        "plt_render_tune": (i32, [vp, C.POINTER(RenderView), u32, u32, u32, C.POINTER(LaunchShape), C.POINTER(C.c_float), vp]),
        "plt_spectral_profile_from_spd": (i32, [C.c_char_p, C.c_float, i32, C.POINTER(SpectralProfile)]),
        "plt_write_exr": (i32, [C.c_char_p, C.POINTER(C.c_float), u32, u32, i32]),
        "plt_render_counters": (i32, [vp, C.POINTER(C.c_uint64), u32]),
        "plt_set_env_map": (i32, [vp, C.POINTER(C.c_float), u32, u32, u32, C.c_float, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
        "plt_clear_env_map": (i32, [vp]),
        "plt_set_analytic_lights": (i32, [vp, vp, u32]),
        "plt_spectral_profiles_from_material": (i32, [C.c_char_p, C.c_char_p, vp, vp]),
        "plt_spectral_profile_for_emitter_type": (i32, [C.c_char_p, C.c_char_p, C.c_float, vp]),
        "plt_env_map_query": (i32, [vp, vp, vp, u32, vp, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class PLTError(RuntimeError):
    def __init__(self, status, where):
        super().__init__("%s failed: %s" % (where, STATUS_NAMES.get(status, status)))
        self.status = status


def check(status, where):
    if status != PLT_OK:
        raise PLTError(status, where)
