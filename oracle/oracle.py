"""ORACLE -- test infrastructure only.  ctypes wrapper of the CPU oracle (oracle/_build/liboracle_plt.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this module, and only as
the checker; the product library never loads it.

Parity status: unpinned by reference tests.  The reference path is Slang shader code that cannot be
compiled here (no slangc, no graphics stack) and the reference ships no PLT tests or golden
vectors; the oracle is a line-by-line C++ restatement of the Slang modules, pinned by physics
known-answer tests (tests/test_oracle_kat.py) and by committed fixtures of its own outputs
(tests/golden/) against regressions.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle_plt.so")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        lib = C.CDLL(LIB)
        vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int
        lib.plto_bsdf_batch.restype = i32
        lib.plto_bsdf_batch.argtypes = [i32, i32, vp, u32, vp, u32, vp, vp, u32, i32]
        lib.plto_bsdf_batch_range.restype = i32
        lib.plto_bsdf_batch_range.argtypes = [i32, i32, vp, u32, vp, u32, vp, vp, u32, i32, C.c_uint64, C.c_uint64]
        lib.plto_trace_brute.restype = None
        lib.plto_trace_brute.argtypes = [vp, u32, vp, vp, vp, vp, u32, i32, vp, vp, vp, vp, i32]
        lib.plto_trace_bvh.restype = None
        lib.plto_trace_bvh.argtypes = [vp, u32, vp, vp, vp, vp, u32, i32, vp, vp, vp, vp, i32]
        lib.plto_set_sr_seed.restype = None
        lib.plto_set_sr_seed.argtypes = [C.c_uint64]
        lib.plto_count_ops.restype = i32
        lib.plto_count_ops.argtypes = [vp, u32, vp, u32, vp, u32, C.POINTER(C.c_double)]
        lib.plto_rng_stream.restype = None
        lib.plto_rng_stream.argtypes = [u32, u32, u32, u32, C.POINTER(C.c_uint32)]
        lib.plto_rng_stream_tiny.restype = None
        lib.plto_rng_stream_tiny.argtypes = [u32, u32, u32, u32, C.POINTER(C.c_uint32)]
        lib.plto_half_to_float.restype = C.c_float
        lib.plto_half_to_float.argtypes = [C.c_uint16]
        lib.plto_rgb_to_spectrum.restype = C.c_float
        lib.plto_rgb_to_spectrum.argtypes = [C.c_float] * 4
        lib.plto_fresnel_dielectric.restype = None
        lib.plto_fresnel_dielectric.argtypes = [C.c_float, C.c_float, C.POINTER(C.c_float)]
        lib.plto_fresnel_conductor.restype = None
        lib.plto_fresnel_conductor.argtypes = [C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double)]
        lib.plto_besselj.restype = C.c_double
        lib.plto_besselj.argtypes = [i32, C.c_double]
        lib.plto_diffract.restype = None
        lib.plto_diffract.argtypes = [C.c_float, C.c_float, C.c_float, i32, i32, C.c_float, C.c_float, C.c_float, C.POINTER(C.c_float)]
        lib.plto_spectral_profile_from_samples.restype = i32
        lib.plto_spectral_profile_from_samples.argtypes = [C.POINTER(C.c_float), C.POINTER(C.c_float), u32, C.c_float, i32, vp]
        _lib = lib
    return _lib


class _Q(C.Structure):
    _fields_ = [("n", C.c_uint32), ("hwss", C.c_uint32), ("rng_offset", C.c_uint32), ("frame", C.c_uint32),
                ("material", C.c_void_p), ("v", C.c_void_p), ("w", C.c_void_p), ("lobe", C.c_void_p),
                ("wavelengths", C.c_void_p), ("stokes", C.c_void_p), ("coherence", C.c_void_p), ("beam_t", C.c_void_p)]


class _R(C.Structure):
    _fields_ = [("stokes", C.c_void_p), ("coherence", C.c_void_p), ("beam_t", C.c_void_p), ("pdf", C.c_void_p),
                ("lambda_pdf", C.c_void_p), ("sample_wo", C.c_void_p), ("sample_pdf", C.c_void_p),
                ("sample_weight", C.c_void_p), ("sample_lobe", C.c_void_p), ("sample_valid", C.c_void_p)]


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def standard_profiles():
    """The workloads' spectral profiles (Au, Ag, Cu, Al eta and k, then D65; the order of
    pltfalcor_gb300.spectra.standard_profiles) built by the oracle's own restatement of
    genSpectralProfile (Scene/SceneBuilder.cpp:911-960), so a CPU-only run of the oracle never loads
    the product library."""
    import sys
    root = os.path.dirname(HERE)
    if root not in sys.path:
        sys.path.insert(0, root)
    from pltfalcor_gb300 import capi, spectra
    lib = load()
    t = spectra.load_tables()
    names = [m + s for m in spectra.METALS for s in (".eta", ".k")] + ["D65"]
    arr = (capi.SpectralProfile * len(names))()
    for i, nm in enumerate(names):
        wl = np.ascontiguousarray(t[nm]["wavelength_nm"], dtype=np.float32)
        v = np.ascontiguousarray(t[nm]["value"], dtype=np.float32)
        st = lib.plto_spectral_profile_from_samples(wl.ctypes.data_as(C.POINTER(C.c_float)), v.ctypes.data_as(C.POINTER(C.c_float)),
                                                    len(wl), 1.0, int(nm == "D65"), C.byref(arr[i]))
        if st != 0:
            raise RuntimeError("oracle spectral profile %s failed with status %d" % (nm, st))
    return arr, {nm: i for i, nm in enumerate(names)}


def make_queries(wl, rng_offset=0):
    q = _Q()
    q.n, q.hwss, q.rng_offset, q.frame = wl.n, wl.hwss, rng_offset, wl.frame
    q.material, q.v, q.w, q.lobe = _p(wl.material), _p(wl.v), _p(wl.w), _p(wl.lobe)
    q.wavelengths, q.stokes, q.coherence, q.beam_t = _p(wl.wavelengths), _p(wl.stokes), _p(wl.coherence), None
    return q


def alloc_results(n, hwss):
    z = lambda k, dt=np.float32: np.zeros(k * n, dt)
    return {"stokes": z(4 * hwss), "coherence": z(4), "pdf": z(1), "lambda_pdf": z(hwss), "sample_wo": z(3),
            "sample_pdf": z(1), "sample_weight": z(1), "sample_lobe": z(1, np.uint32), "sample_valid": z(1, np.uint32)}


def results_struct(res):
    r = _R()
    for k in res:
        setattr(r, k, _p(res[k]))
    return r


def run(wl, ops=None, precision=32, threads=0, fp64_multilayer=False, begin=0, end=None, res=None, sr_seed=None,
        fp64_conductor_grazing=False):
    """Runs the oracle over queries [begin, end) of workload `wl`; returns the results dict.
    precision: 32 (FP32), 64 (FP64) or 16 (FP32 with random rounding, seed `sr_seed`);
    fp64_multilayer / fp64_conductor_grazing: the FP32 oracle's twins of the library's
    PLT_OPTION_FP64_MULTILAYER / PLT_OPTION_FP64_CONDUCTOR_GRAZING."""
    lib = load()
    if precision == 16:
        lib.plto_set_sr_seed(1 if sr_seed is None else sr_seed)
    ops = wl.ops if ops is None else ops
    end = wl.n if end is None else end
    q = make_queries(wl)
    res = alloc_results(wl.n, wl.hwss) if res is None else res
    r = results_struct(res)
    recs = np.ascontiguousarray(wl.records)
    prof = wl.profiles
    flags = (0x1 if fp64_multilayer else 0) | (0x10 if fp64_conductor_grazing else 0)
    st = lib.plto_bsdf_batch_range(precision, flags, C.c_void_p(recs.ctypes.data), len(recs),
                                   C.cast(prof, C.c_void_p) if prof is not None else None, len(prof) if prof is not None else 0,
                                   C.byref(q), C.byref(r), ops, threads, begin, end)
    if st != 0:
        raise RuntimeError("oracle batch failed with status %d" % st)
    return res


def count_ops(wl, ops=None):
    """Mean (fp, sfu, div, count) per material type of the op-counting build."""
    lib = load()
    ops = wl.ops if ops is None else ops
    q = make_queries(wl)
    out = (C.c_double * (12 * 4))()
    recs = np.ascontiguousarray(wl.records)
    prof = wl.profiles
    st = lib.plto_count_ops(C.c_void_p(recs.ctypes.data), len(recs), C.cast(prof, C.c_void_p) if prof is not None else None,
                            len(prof) if prof is not None else 0, C.byref(q), ops, out)
    if st != 0:
        raise RuntimeError("oracle count failed with status %d" % st)
    a = np.frombuffer(out, dtype=np.float64).reshape(12, 4)
    return {t: {"fp": a[t, 0], "sfu": a[t, 1], "div": a[t, 2], "count": int(a[t, 3])} for t in range(12) if a[t, 3] > 0}


def trace_brute(tri_verts, origin, direction, tmin=None, tmax=None, any_hit=False, threads=0, bvh=False):
    """Brute-force closest hit (prim, t, bary) or occlusion over all triangles ([n_tri][9] vertices);
    bvh=True runs the same query through the oracle's BVH (identical results)."""
    lib = load()
    fn = lib.plto_trace_bvh if bvh else lib.plto_trace_brute
    tv = np.ascontiguousarray(tri_verts, np.float32)
    o = np.ascontiguousarray(origin, np.float32)
    d = np.ascontiguousarray(direction, np.float32)
    n = len(o) // 3
    p = lambda a: None if a is None else C.c_void_p(np.ascontiguousarray(a, np.float32).ctypes.data)
    t0 = None if tmin is None else np.ascontiguousarray(tmin, np.float32)
    t1 = None if tmax is None else np.ascontiguousarray(tmax, np.float32)
    if any_hit:
        occ = np.zeros(n, np.uint32)
        fn(C.c_void_p(tv.ctypes.data), len(tv), C.c_void_p(o.ctypes.data), C.c_void_p(d.ctypes.data), p(t0), p(t1),
           n, 1, None, None, None, C.c_void_p(occ.ctypes.data), threads or os.cpu_count())
        return occ
    prim = np.zeros(n, np.uint32)
    t = np.zeros(n, np.float32)
    bary = np.zeros(2 * n, np.float32)
    fn(C.c_void_p(tv.ctypes.data), len(tv), C.c_void_p(o.ctypes.data), C.c_void_p(d.ctypes.data), p(t0), p(t1),
       n, 0, C.c_void_p(prim.ctypes.data), C.c_void_p(t.ctypes.data), C.c_void_p(bary.ctypes.data), None,
       threads or os.cpu_count())
    return prim, t, bary


def rng_stream(px, py, frame, count, tiny=False):
    """The generator's first `count` 32-bit outputs for (pixel, frame): UniformSampleGenerator, or
    TinyUniformSampleGenerator with tiny=True."""
    out = (C.c_uint32 * count)()
    (load().plto_rng_stream_tiny if tiny else load().plto_rng_stream)(px, py, frame, count, out)
    return np.frombuffer(out, dtype=np.uint32).copy()


class _Scene(C.Structure):
    _fields_ = [("n_vertices", C.c_uint32), ("n_triangles", C.c_uint32), ("n_materials", C.c_uint32), ("n_profiles", C.c_uint32),
                ("positions", C.c_void_p), ("normals", C.c_void_p), ("tangents", C.c_void_p), ("indices", C.c_void_p),
                ("tri_material", C.c_void_p), ("tri_instance", C.c_void_p), ("materials", C.c_void_p), ("profiles", C.c_void_p),
                ("proposal_params", C.c_void_p), ("env", C.c_void_p), ("lights", C.c_void_p), ("n_lights", C.c_uint32)]


class _Env(C.Structure):
    _fields_ = [("rgb", C.c_void_p), ("width", C.c_uint32), ("height", C.c_uint32), ("intensity", C.c_float),
                ("tint", C.c_float * 3), ("rotation_deg", C.c_float * 3)]


def _env_struct(env):
    """env: dict(rgb=[height][width][3 or 4] array, intensity=1, tint=(1, 1, 1), rotation=(0, 0, 0))."""
    if env is None:
        return None, None
    rgb = np.ascontiguousarray(np.asarray(env["rgb"], np.float32)[..., :3])
    e = _Env(rgb.ctypes.data, rgb.shape[1], rgb.shape[0], float(env.get("intensity", 1.0)),
             (C.c_float * 3)(*[float(x) for x in env.get("tint", (1.0, 1.0, 1.0))]),
             (C.c_float * 3)(*[float(x) for x in env.get("rotation", (0.0, 0.0, 0.0))]))
    return e, rgb


def env_query(env, u, dirs=None):
    """The oracle's environment sampler on given inputs: [n][12] as plt_env_map_query."""
    lib = load()
    lib.plto_env_query.restype = C.c_int
    lib.plto_env_query.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p]
    e, keep = _env_struct(env)
    u = np.ascontiguousarray(u, np.float32).reshape(-1, 2)
    d = None if dirs is None else np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
    out = np.zeros((len(u), 12), np.float32)
    st = lib.plto_env_query(C.addressof(e), u.ctypes.data, None if d is None else d.ctypes.data, len(u), out.ctypes.data)
    if st != 0:
        raise RuntimeError("plto_env_query failed: %d" % st)
    return out


def _scene_struct(scene, profiles, proposal_params=None, env=None, lights=None):
    keep = [np.ascontiguousarray(scene.vertices, np.float32), np.ascontiguousarray(scene.normals, np.float32),
            np.ascontiguousarray(scene.indices, np.uint32), np.ascontiguousarray(scene.tri_material, np.uint32),
            np.ascontiguousarray(scene.records)]
    tan = None if getattr(scene, "tangents", None) is None else np.ascontiguousarray(scene.tangents, np.float32)
    inst = None if getattr(scene, "tri_instance", None) is None else np.ascontiguousarray(scene.tri_instance, np.uint32)
    s = _Scene(len(keep[0]), len(keep[2]), len(keep[4]), len(profiles) if profiles is not None else 0,
               keep[0].ctypes.data, keep[1].ctypes.data, None if tan is None else tan.ctypes.data, keep[2].ctypes.data,
               keep[3].ctypes.data, None if inst is None else inst.ctypes.data, keep[4].ctypes.data,
               C.cast(profiles, C.c_void_p) if profiles is not None else None)
    pp = None if proposal_params is None else np.ascontiguousarray(proposal_params, np.float32)
    s.proposal_params = None if pp is None else pp.ctypes.data
    e, erg = _env_struct(env)
    s.env = None if e is None else C.addressof(e)
    larr = None
    if lights:
        larr = (type(lights[0]) * len(lights))(*lights)
        s.lights, s.n_lights = C.addressof(larr), len(lights)
    return s, (keep, tan, inst, profiles, pp, e, erg, larr)


def render(scene, profiles, camera, options, width, height, frame=0, threads=0, records=False, frames=1, proposal_params=None,
           env=None, lights=None):
    """FP32 oracle render of one frame: rgb [height][width][3]; with records=True also per-path bounce
    records (prim, lobe, flags) [height*width][max_bounces+1] and stats (paths, shadow rays, evals).
    `profiles` is a ctypes array of plt_spectral_profile, `camera`/`options` the ctypes structs of
    include/plt_gb300.h; `proposal_params` (11488 floats) the network of learned_proposal renders;
    `env` the environment light (dict of rgb, intensity, tint, rotation)."""
    lib = load()
    if not hasattr(lib, "_render_sig"):
        lib.plto_render.restype = C.c_int
        lib.plto_render.argtypes = [C.c_void_p] * 3 + [C.c_uint32] * 4 + [C.c_int] + [C.c_void_p] * 5
        lib.plto_light_table.restype = C.c_uint32
        lib.plto_light_table.argtypes = [C.c_void_p] * 4
        lib._render_sig = True
    s, keep = _scene_struct(scene, profiles, proposal_params, env, lights)
    rgb = np.zeros((height, width, 3), np.float32)
    nb = options.max_bounces + 1
    recs = [np.zeros((height * width, nb), np.uint32) for _ in range(3)] if records else [None] * 3
    stats = np.zeros(3, np.uint64)
    st = lib.plto_render(C.addressof(s), C.addressof(camera), C.addressof(options), width, height, frame, frames,
                         threads or os.cpu_count(), rgb.ctypes.data, *[None if r is None else r.ctypes.data for r in recs],
                         stats.ctypes.data)
    if st != 0:
        raise RuntimeError("plto_render failed: %d" % st)
    return (rgb, recs, stats) if records else rgb


def light_table(scene, profiles):
    """(alias [n][2] uint32, light triangles [n], inverse weight sum) as the oracle builds them."""
    lib = load()
    if not hasattr(lib, "_render_sig"):
        lib.plto_light_table.restype = C.c_uint32
        lib.plto_light_table.argtypes = [C.c_void_p] * 4
    s, keep = _scene_struct(scene, profiles)
    n = lib.plto_light_table(C.addressof(s), None, None, None)
    alias = np.zeros((n, 2), np.uint32)
    tris = np.zeros(n, np.uint32)
    inv = C.c_float(0)
    lib.plto_light_table(C.addressof(s), alias.ctypes.data, tris.ctypes.data, C.byref(inv))
    return alias, tris, inv.value


def _mlp_sig(lib):
    if not hasattr(lib, "_mlp_sig"):
        lib.plto_mlp_forward.restype = None
        lib.plto_mlp_forward.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_void_p]
        lib.plto_mlp_gradient.restype = C.c_double
        lib.plto_mlp_gradient.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_int, C.c_void_p]
        lib._mlp_sig = True


def mlp_forward(params, x_bits, round_bf16=True):
    """Proposal network outputs [n][32] for bf16 feature rows x_bits [n][16] (uint16)."""
    lib = load()
    _mlp_sig(lib)
    p = np.ascontiguousarray(params, np.float32)
    x = np.ascontiguousarray(x_bits, np.uint16)
    n = len(x)
    out = np.zeros((n, 32), np.float32)
    lib.plto_mlp_forward(p.ctypes.data, x.ctypes.data, n, int(round_bf16), out.ctypes.data)
    return out


def mlp_gradient(params, target, weight, x_bits=None, x_f64=None, round_bf16=True):
    """(mean weighted mixture NLL, gradient [11488]) of a batch; features as bf16 bits or float64."""
    lib = load()
    _mlp_sig(lib)
    p = np.ascontiguousarray(params, np.float32)
    t = np.ascontiguousarray(target, np.float32)
    w = np.ascontiguousarray(weight, np.float32)
    xb = None if x_bits is None else np.ascontiguousarray(x_bits, np.uint16)
    xf = None if x_f64 is None else np.ascontiguousarray(x_f64, np.float64)
    n = len(w)
    g = np.zeros(11488, np.float64)
    loss = lib.plto_mlp_gradient(p.ctypes.data, None if xb is None else xb.ctypes.data, None if xf is None else xf.ctypes.data,
                                 t.ctypes.data, w.ctypes.data, n, int(round_bf16), g.ctypes.data)
    return loss, g
