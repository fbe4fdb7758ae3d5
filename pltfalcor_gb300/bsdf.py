"""Python mirror of the batched IMaterialInstance interface over libplt_gb300.so.

`PLTContext` owns one C-ABI context (plt_create / plt_destroy).  Queries and results are CUDA
tensors (torch is only the device-memory and stream plumbing); every call goes through the C ABI
and raises PLTError on a non-OK status.  Method names follow the reference interface:
eval / sample / pdf / lambdaPdf (Source/Falcor/Rendering/Materials/IMaterialInstance.slang:122-184
in ssteinberg/PLTFalcor).
"""
import ctypes as C

import numpy as np

from . import capi


def _ptr(t):
    return None if t is None else C.c_void_p(t.data_ptr())


class DeviceBatch:
    """A query batch resident on the GPU (or, with device="cpu", in host memory, pinned when pin is
    set: the buffers of plt_bsdf_batch_host), with result buffers for the requested ops."""

    def __init__(self, workload, device="cuda", pin=False, results=True):
        import torch
        self.workload = workload
        self.n, self.hwss = workload.n, workload.hwss
        d = torch.device(device)
        self._pin_host = pin and d.type == "cpu"

        def up(a, dt):
            if a is None:
                return None
            t = torch.from_numpy(a)
            if dt is not None:
                t = t.view(dt)
            if self._pin_host:
                return t.pin_memory()
            return t.to(d, non_blocking=pin)
        self.material = up(workload.material.view(np.int32), None)
        self.v = up(workload.v, None)
        self.w = up(workload.w, None)
        self.lobe = up(None if workload.lobe is None else workload.lobe.view(np.int32), None)
        self.wavelengths = up(workload.wavelengths, None)
        self.stokes = up(workload.stokes, None)
        self.coherence = up(workload.coherence, None)
        self.beam_t = None
        if results:
            self.alloc_results(d)

    def alloc_results(self, d):
        import torch
        n, h = self.n, self.hwss
        pin = getattr(self, "_pin_host", False)
        f = lambda k: torch.zeros(k * n, dtype=torch.float32, device=d, pin_memory=pin)
        self.out_stokes = f(4 * h)
        self.out_coherence = f(4)
        self.out_beam_t = None
        self.out_pdf = f(1)
        self.out_lambda_pdf = f(h)
        self.out_sample_wo = f(3)
        self.out_sample_pdf = f(1)
        self.out_sample_weight = f(1)
        self.out_sample_lobe = torch.zeros(n, dtype=torch.int32, device=d, pin_memory=pin)
        self.out_sample_valid = torch.zeros(n, dtype=torch.int32, device=d, pin_memory=pin)

    def queries(self, rng_offset=0, frame=None):
        """plt_bsdf_queries over the resident planes (plane stride = n)."""
        q = capi.BsdfQueries()
        q.n = self.n
        q.hwss = self.hwss
        q.rng_offset = rng_offset
        q.frame = self.workload.frame if frame is None else frame
        q.material, q.v, q.w = _ptr(self.material), _ptr(self.v), _ptr(self.w)
        q.lobe = _ptr(self.lobe)
        q.wavelengths, q.stokes, q.coherence = _ptr(self.wavelengths), _ptr(self.stokes), _ptr(self.coherence)
        q.beam_t = _ptr(self.beam_t)
        return q

    def results(self, ops):
        r = capi.BsdfResults()
        if ops & capi.OP_EVAL:
            r.stokes, r.coherence, r.beam_t = _ptr(self.out_stokes), _ptr(self.out_coherence), _ptr(self.out_beam_t)
        if ops & capi.OP_PDF:
            r.pdf = _ptr(self.out_pdf)
        if ops & capi.OP_LAMBDA_PDF:
            r.lambda_pdf = _ptr(self.out_lambda_pdf)
        if ops & capi.OP_SAMPLE:
            r.sample_wo, r.sample_pdf = _ptr(self.out_sample_wo), _ptr(self.out_sample_pdf)
            r.sample_weight, r.sample_lobe = _ptr(self.out_sample_weight), _ptr(self.out_sample_lobe)
            r.sample_valid = _ptr(self.out_sample_valid)
        return r

    def fetch(self):
        """Results as host numpy arrays (same keys as the oracle's results)."""
        g = lambda t: t.cpu().numpy()
        return {"stokes": g(self.out_stokes), "coherence": g(self.out_coherence), "pdf": g(self.out_pdf),
                "lambda_pdf": g(self.out_lambda_pdf), "sample_wo": g(self.out_sample_wo),
                "sample_pdf": g(self.out_sample_pdf), "sample_weight": g(self.out_sample_weight),
                "sample_lobe": g(self.out_sample_lobe).view(np.uint32), "sample_valid": g(self.out_sample_valid).view(np.uint32)}


class PLTContext:
    """One context on the current CUDA device: material table, spectral tables, batched BSDF ops."""

    def __init__(self, options=None, fp64_multilayer=False):
        self.lib = capi.load_library()
        opts = capi.Options()
        self.lib.plt_options_default(C.byref(opts))
        if options:
            for k, val in options.items():
                setattr(opts, k, val)
        if fp64_multilayer:
            opts.flags |= capi.OPTION_FP64_MULTILAYER
        h = C.c_void_p()
        capi.check(self.lib.plt_create(C.byref(opts), C.byref(h)), "plt_create")
        self.handle = h

    def close(self):
        if self.handle:
            self.lib.plt_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_spectral_profiles(self, profiles):
        capi.check(self.lib.plt_set_spectral_profiles(self.handle, profiles, len(profiles)), "plt_set_spectral_profiles")

    def set_materials(self, records):
        recs = np.ascontiguousarray(records)
        capi.check(self.lib.plt_set_materials(self.handle, recs.ctypes.data_as(C.POINTER(capi.MaterialRecord)), len(recs)),
                   "plt_set_materials")

    def batch(self, queries, results, ops, stream=None):
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        capi.check(self.lib.plt_bsdf_batch(self.handle, C.byref(queries), C.byref(results), ops, s), "plt_bsdf_batch")

    def batch_host(self, queries, results, ops, stream=None):
        """plt_bsdf_batch_host: queries and results in host memory (a DeviceBatch on "cpu")."""
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        capi.check(self.lib.plt_bsdf_batch_host(self.handle, C.byref(queries), C.byref(results), ops, s), "plt_bsdf_batch_host")

    def eval(self, q, r, stream=None):
        self.batch(q, r, capi.OP_EVAL, stream)

    def pdf(self, q, r, stream=None):
        self.batch(q, r, capi.OP_PDF, stream)

    def sample(self, q, r, stream=None):
        self.batch(q, r, capi.OP_SAMPLE, stream)

    def lambdaPdf(self, q, r, stream=None):
        self.batch(q, r, capi.OP_LAMBDA_PDF, stream)

    # ---- scene and ray queries (replace the DXR acceleration structure and TraceRay) ----
    def set_scene(self, vertices, indices, tri_material=None):
        v = np.ascontiguousarray(vertices, np.float32)
        f = np.ascontiguousarray(indices, np.uint32)
        m = None if tri_material is None else np.ascontiguousarray(tri_material, np.uint32)
        capi.check(self.lib.plt_set_scene(self.handle, C.c_void_p(v.ctypes.data), len(v), C.c_void_p(f.ctypes.data), len(f),
                                          None if m is None else C.c_void_p(m.ctypes.data)), "plt_set_scene")

    def scene_stats(self):
        out = (C.c_uint32 * 4)()
        capi.check(self.lib.plt_scene_stats(self.handle, out), "plt_scene_stats")
        return {"nodes": out[0], "leaves": out[1], "max_depth": out[2], "triangles": out[3]}

    @staticmethod
    def rays(origin, direction, tmin=None, tmax=None, stats=None):
        r = capi.Rays()
        r.n = origin.numel() // 3
        r.origin, r.dir = _ptr(origin), _ptr(direction)
        r.tmin, r.tmax, r.stats = _ptr(tmin), _ptr(tmax), _ptr(stats)
        return r

    def trace_closest(self, rays, prim, t=None, bary=None, stream=None):
        h = capi.Hits()
        h.prim, h.t, h.bary = _ptr(prim), _ptr(t), _ptr(bary)
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        capi.check(self.lib.plt_trace_closest(self.handle, C.byref(rays), C.byref(h), s), "plt_trace_closest")

    def trace_any(self, rays, occluded, stream=None):
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        capi.check(self.lib.plt_trace_any(self.handle, C.byref(rays), _ptr(occluded), s), "plt_trace_any")

    def check_status(self, stream=None):
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        return self.lib.plt_check_status(self.handle, s)

    def last_bounds_violation(self):
        """(site, index, bound) of the first violation the last check_status reported as
        PLT_BOUNDS_VIOLATION (a -DPLT_BOUNDS_CHECK=1 build), zeros when none."""
        out = (C.c_uint32 * 3)()
        capi.check(self.lib.plt_last_bounds_violation(self.handle, out), "plt_last_bounds_violation")
        return tuple(int(x) for x in out)

    # ---- PLTPT render pass ----
    def set_scene_shading(self, normals, tangents=None, tri_instance=None):
        n = np.ascontiguousarray(normals, np.float32)
        t = None if tangents is None else np.ascontiguousarray(tangents, np.float32)
        g = None if tri_instance is None else np.ascontiguousarray(tri_instance, np.uint32)
        capi.check(self.lib.plt_set_scene_shading(self.handle, C.c_void_p(n.ctypes.data), None if t is None else C.c_void_p(t.ctypes.data),
                                                  len(n), None if g is None else C.c_void_p(g.ctypes.data)), "plt_set_scene_shading")

    def load_scene(self, scene, profiles):
        """Spectral profiles, materials, geometry and shading attributes of a scene.Scene."""
        self.set_spectral_profiles(profiles)
        self.set_materials(scene.records)
        self.set_scene(scene.vertices, scene.indices, scene.tri_material)
        self.set_scene_shading(scene.normals, scene.tangents, getattr(scene, "tri_instance", None))

    def render(self, camera, width, height, out_rgba, frame_begin=0, frame_count=1, stream=None):
        """plt_render into the device tensor out_rgba [height][width][4] (float32)."""
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        capi.check(self.lib.plt_render(self.handle, C.byref(camera), width, height, frame_begin, frame_count, _ptr(out_rgba), s),
                   "plt_render")

    # ---- scene sets ----
    def add_scene(self, scene, material_offset=0):
        """Appends a scene.Scene (geometry + shading) to the context's scene set; its tri_material
        indices are shifted by material_offset into the context's material table.  Returns the index."""
        keep = [np.ascontiguousarray(scene.vertices, np.float32), np.ascontiguousarray(scene.indices, np.uint32),
                np.ascontiguousarray(scene.tri_material + np.uint32(material_offset), np.uint32),
                np.ascontiguousarray(scene.normals, np.float32)]
        tan = None if scene.tangents is None else np.ascontiguousarray(scene.tangents, np.float32)
        inst = None if getattr(scene, "tri_instance", None) is None else np.ascontiguousarray(scene.tri_instance, np.uint32)
        d = capi.SceneDesc(keep[0].ctypes.data, len(keep[0]), keep[1].ctypes.data, len(keep[1]), keep[2].ctypes.data,
                           keep[3].ctypes.data, None if tan is None else tan.ctypes.data, None if inst is None else inst.ctypes.data)
        out = C.c_uint32(0)
        capi.check(self.lib.plt_add_scene(self.handle, C.byref(d), C.byref(out)), "plt_add_scene")
        return out.value

    def clear_scenes(self):
        capi.check(self.lib.plt_clear_scenes(self.handle), "plt_clear_scenes")

    def set_env_map(self, rgb, intensity=1.0, tint=(1.0, 1.0, 1.0), rotation=(0.0, 0.0, 0.0)):
        """plt_set_env_map: rgb is a [height][width][3 or 4] float array (linear lat-long map)."""
        a = np.ascontiguousarray(np.asarray(rgb, np.float32))
        if a.ndim != 3 or a.shape[2] not in (3, 4):
            raise ValueError("env map must be [height][width][3 or 4]")
        t = (C.c_float * 3)(*[float(x) for x in tint])
        r = (C.c_float * 3)(*[float(x) for x in rotation])
        capi.check(self.lib.plt_set_env_map(self.handle, a.ctypes.data_as(C.POINTER(C.c_float)), a.shape[1], a.shape[0],
                                            a.shape[2], float(intensity), t, r), "plt_set_env_map")

    def set_analytic_lights(self, lights):
        """plt_set_analytic_lights from a list of capi.AnalyticLight (scene.*_light helpers)."""
        arr = (capi.AnalyticLight * max(1, len(lights)))(*lights)
        capi.check(self.lib.plt_set_analytic_lights(self.handle, arr if lights else None, len(lights)), "plt_set_analytic_lights")

    def clear_env_map(self):
        capi.check(self.lib.plt_clear_env_map(self.handle), "plt_clear_env_map")

    def env_map_query(self, u, dirs=None, stream=None):
        """plt_env_map_query on device tensors u [n][2] (and dirs [n][3]): returns [n][12] on the device."""
        import torch
        n = u.shape[0]
        out = torch.empty((n, 12), dtype=torch.float32, device=u.device)
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        capi.check(self.lib.plt_env_map_query(self.handle, C.c_void_p(u.data_ptr()),
                                              None if dirs is None else C.c_void_p(dirs.data_ptr()), n,
                                              C.c_void_p(out.data_ptr()), s), "plt_env_map_query")
        return out

    def render_scenes(self, views, frame_begin=0, frame_count=1, stream=None):
        """plt_render_scenes: views is a list of (scene index, camera, width, height, out tensor [h][w][4])."""
        arr = self._views(views)
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        capi.check(self.lib.plt_render_scenes(self.handle, arr, len(views), frame_begin, frame_count, s), "plt_render_scenes")

    def _views(self, views):
        arr = (capi.RenderView * len(views))()
        for i, (sid, cam, w, h, out) in enumerate(views):
            arr[i].scene, arr[i].width, arr[i].height = sid, w, h
            arr[i].camera = cam
            arr[i].out_rgba = _ptr(out)
        return arr

    def set_launch_shape(self, wave_paths=0, segment=0, solve=0, walk=0, path_order=0):
        sh = capi.LaunchShape(wave_paths, segment, solve, walk, path_order)
        capi.check(self.lib.plt_set_launch_shape(self.handle, C.byref(sh)), "plt_set_launch_shape")

    def launch_shape(self):
        sh = capi.LaunchShape()
        capi.check(self.lib.plt_get_launch_shape(self.handle, C.byref(sh)), "plt_get_launch_shape")
        return {"wave_paths": sh.wave_paths, "segment": sh.segment_blocks_per_sm, "solve": sh.solve_blocks_per_sm,
                "walk": sh.walk_blocks_per_sm, "path_order": sh.path_order}

    def render_tune(self, views, frame=0, frames=1, stream=None):
        """plt_render_tune over views (as render_scenes); returns (shape dict, ms per frame)."""
        arr = self._views(views)
        sh, ms = capi.LaunchShape(), C.c_float(0)
        s = C.c_void_p(stream.cuda_stream) if stream is not None else None
        capi.check(self.lib.plt_render_tune(self.handle, arr, len(views), frame, frames, C.byref(sh), C.byref(ms), s), "plt_render_tune")
        return self.launch_shape(), ms.value

    def render_bounces(self, npix, max_bounces):
        """Bounce records of the last frame: (prim, lobe, flags), each [npix][max_bounces+1] uint32."""
        out = [np.zeros((npix, max_bounces + 1), np.uint32) for _ in range(3)]
        capi.check(self.lib.plt_render_bounces(self.handle, *[C.c_void_p(a.ctypes.data) for a in out]), "plt_render_bounces")
        return out

    # ---- learned MIS proposal ----
    def proposal_init(self, seed=0):
        capi.check(self.lib.plt_proposal_init(self.handle, seed), "plt_proposal_init")

    def proposal_params(self):
        out = np.zeros(capi.PROPOSAL_PARAMS, np.float32)
        capi.check(self.lib.plt_proposal_get_params(self.handle, out.ctypes.data_as(C.POINTER(C.c_float))), "plt_proposal_get_params")
        return out

    def proposal_set_params(self, params):
        p = np.ascontiguousarray(params, np.float32)
        capi.check(self.lib.plt_proposal_set_params(self.handle, p.ctypes.data_as(C.POINTER(C.c_float))), "plt_proposal_set_params")

    def proposal_generate(self, n, seed, device="cuda"):
        """Training batch from the exact samplers: (x bf16 bits as int16 [n][16], target [n][2], weight [n])."""
        import torch
        x = torch.zeros((n, 16), dtype=torch.int16, device=device)
        t = torch.zeros((n, 2), dtype=torch.float32, device=device)
        w = torch.zeros(n, dtype=torch.float32, device=device)
        capi.check(self.lib.plt_proposal_generate(self.handle, n, seed, _ptr(x), _ptr(t), _ptr(w), None), "plt_proposal_generate")
        return x, t, w

    def proposal_gradient(self, x, t, w):
        import torch
        g = torch.zeros(capi.PROPOSAL_PARAMS, dtype=torch.float32, device=x.device)
        loss = torch.zeros(1, dtype=torch.float32, device=x.device)
        capi.check(self.lib.plt_proposal_gradient(self.handle, len(w), _ptr(x), _ptr(t), _ptr(w), _ptr(g), _ptr(loss), None),
                   "plt_proposal_gradient")
        return float(loss.item()), g

    def proposal_forward(self, x):
        import torch
        out = torch.zeros((x.shape[0], 32), dtype=torch.float32, device=x.device)
        capi.check(self.lib.plt_proposal_forward(self.handle, x.shape[0], _ptr(x), _ptr(out), None), "plt_proposal_forward")
        return out

    def proposal_adam_step(self, grad, lr=1e-3):
        """One Adam step of the proposal with a device gradient [11488] (e.g. a rank-averaged one)."""
        capi.check(self.lib.plt_proposal_adam_step(self.handle, _ptr(grad), lr, None), "plt_proposal_adam_step")

    def proposal_train(self, steps, batch=65536, lr=1e-3, seed=1):
        hist = np.zeros(steps, np.float32)
        capi.check(self.lib.plt_proposal_train(self.handle, steps, batch, lr, seed, hist.ctypes.data_as(C.POINTER(C.c_float)), None),
                   "plt_proposal_train")
        return hist

    def render_counters(self):
        out = (C.c_uint64 * 5)()
        capi.check(self.lib.plt_render_counters(self.handle, out, 5), "plt_render_counters")
        return {"paths": out[0], "bounces": out[1], "shadow_rays": out[2], "bsdf_evals": out[3], "traversal_bytes": out[4]}

    def render_stats(self):
        out = (C.c_uint64 * 4)()
        capi.check(self.lib.plt_render_stats(self.handle, out), "plt_render_stats")
        return {"paths": out[0], "bounces": out[1], "shadow_rays": out[2], "bsdf_evals": out[3]}
