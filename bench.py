"""Benchmark of the PLT BSDF hot path on GB300.

Workload: the mixed-material batch -- 2^22 eval + sample + pdf queries split equally over the eight
PLT material types (dielectric, conductor, coated opaque dielectric, coated conductor, grated
opaque dielectric, grated conductor, birefringent thin dielectric, multilayer stack) in shuffled
order, HWSS 1, seed 1 (pltfalcor_gb300/workloads.py).  A step is one fused plt_bsdf_batch launch
over the whole batch.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

value: queries/s with inputs resident in HBM (CUDA events on the launching stream; inputs and
outputs together exceed L2, so no flush is needed).  e2e: the same metric through the C ABI with
host (pinned) buffers (plt_bsdf_batch_host) -- every step copies the inputs host->device and all
outputs device->host, in chunks whose copies overlap the kernels; consecutive steps are independent
batches on two alternating streams (two host buffer sets), so one step's input copies overlap the
previous step's output copies.
The reference arm (--impl reference) times the CPU restatement of the reference's BSDF code (the
reference's own path is Slang shader code with no CPU build) on all host threads.
Under torchrun each rank processes its own batch (weak scaling); rank 0 prints one JSON line.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_DEFAULT = 1 << 22
METRIC = "PLT BSDF queries/s (eval+sample+pdf, 8 PLT materials)"
WORKLOAD = ("mixed_material_batch: 2^22 eval+sample+pdf queries over 8 PLT material types (2^19 each, shuffled), "
            "HWSS 1, 32768 random materials, seed 1")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 100 ms while running."""

    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for nm, v in zip(names, r[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(n_sample=1 << 18, seconds=10.0, threads=None):
    """The oracle (CPU restatement of the reference BSDF code, FP32, OpenMP) on a bounded sample of
    the same workload: repeated 2^18-query slices until `seconds` have elapsed."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from pltfalcor_gb300 import spectra
    from pltfalcor_gb300 import workloads as W
    threads = threads or os.cpu_count()
    prof, _ = spectra.standard_profiles()
    wl = W.mixed_material_batch(n=n_sample, profiles=prof)
    oracle.run(wl, threads=threads)  # warm-up
    done, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < seconds:
        oracle.run(wl, threads=threads)
        done += wl.n
    dt = time.perf_counter() - t0
    return {"value": done / dt, "unit": "queries/s", "cores": threads, "kind": "port",
            "sample": "%d queries (%d-query slices of the mixed-material batch, seed 1) in %.1f s, FP32 oracle, OpenMP" % (done, n_sample, dt)}


def camera_rays(res, pos, look, up, fov_deg):
    """Pinhole primary rays through pixel centres (res x res), SoA planes."""
    import numpy as np
    w = np.asarray(look, np.float64) - np.asarray(pos, np.float64)
    w /= np.linalg.norm(w)
    u = np.cross(w, up)
    u /= np.linalg.norm(u)
    v = np.cross(u, w)
    th = np.tan(np.radians(fov_deg) / 2)
    px = (np.arange(res) + 0.5) / res * 2 - 1
    X, Y = np.meshgrid(px, -px)
    d = w[:, None] + th * (X.ravel()[None, :] * u[:, None] + Y.ravel()[None, :] * v[:, None])
    d /= np.linalg.norm(d, axis=0, keepdims=True)
    o = np.repeat(np.asarray(pos, np.float64)[:, None], res * res, axis=1)
    return np.ascontiguousarray(o.astype(np.float32).reshape(-1)), np.ascontiguousarray(d.astype(np.float32).reshape(-1))


def trace_bench(ctx, dev, stream, steps, warmup):
    """Closest-hit traversal on the 1.04 M-triangle procedural scene: 1024^2 pinhole primary rays
    and 2^20 rays from random points in random directions.  Algorithmic bytes per ray = BVH node
    visits x 64 B + triangle tests x 48 B, counted by the kernel in a separate untimed launch."""
    import torch
    from pltfalcor_gb300 import scene as S
    sc = S.procedural_scene()
    t0 = time.perf_counter()
    ctx.set_scene(sc.vertices, sc.indices, sc.tri_material)
    build_s = time.perf_counter() - t0
    st = ctx.scene_stats()
    out = {"scene": "procedural room: box + 200 level-4 icospheres + 500 quads + light + glass sphere (seed 2)",
           "triangles": sc.n_tris, "bvh_nodes": st["nodes"], "bvh_max_depth": st["max_depth"], "bvh_build_s_host": build_s}
    sets = {"primary_1024x1024": camera_rays(1024, (0.0, -9.5, 0.0), (0.0, 0.0, 0.0), (0.0, 0.0, 1.0), 60.0),
            "random_1M": S.random_rays(1 << 20, 13, sc.bounds)}
    for name, (o, d) in sets.items():
        n = len(o) // 3
        go, gd = torch.from_numpy(o).to(dev), torch.from_numpy(d).to(dev)
        prim = torch.zeros(n, dtype=torch.int32, device=dev)
        t = torch.zeros(n, dtype=torch.float32, device=dev)
        bary = torch.zeros(2 * n, dtype=torch.float32, device=dev)
        stats = torch.zeros(2, dtype=torch.int64, device=dev)
        ctx.trace_closest(ctx.rays(go, gd, None, None, stats), prim, t, bary, stream)
        torch.cuda.synchronize()
        nv, tt = [int(x) for x in stats.cpu()]
        r = ctx.rays(go, gd)
        for _ in range(warmup):
            ctx.trace_closest(r, prim, t, bary, stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            ctx.trace_closest(r, prim, t, bary, stream)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        bpr = (nv * 64 + tt * 48) / n + 12 * 2 + 16  # + ray in (24 B) + hit out (prim, t, bary: 16 B)
        out[name] = {"rays": n, "ms_per_launch": ms, "rays_per_s": n / (ms * 1e-3), "node_visits_per_ray": nv / n,
                     "tri_tests_per_ray": tt / n, "algorithmic_bytes_per_ray": bpr,
                     "achieved_gbs": bpr * n / (ms * 1e-3) / 1e9, "miss_frac": float((prim == -1).float().mean().item())}
    return out


def render_bench(dev, stream, frames, warmup, cpu_seconds=0.0, size=1024):
    """PLTPT render pass (sample + solve) on the 1.04 M-triangle procedural room: 1024^2 paths per
    frame, max depth 8, HWSS 4 with spectral MIS, NEE + MIS with manifold walks, Russian roulette,
    power-sampled emissive light; one frame per launch sequence, `frames` frames timed with CUDA events.  e2e
    adds the device-to-host read of the accumulated image.  The CPU figure is the oracle's
    restatement of both passes (OpenMP, its own BVH) on a 128^2 image of the same view."""
    import ctypes as C
    import numpy as np
    import torch
    from pltfalcor_gb300 import scene as S, spectra
    from pltfalcor_gb300.bsdf import PLTContext
    prof, _ = spectra.standard_profiles()
    sc = S.procedural_scene()
    opts = {"max_bounces": 8, "hwss": 4, "do_mnee": 1, "mnee_max_occluders": 2, "mnee_max_iterations": 60,
            "mnee_solver_threshold": 5e-5}
    ctx = PLTContext(opts)
    ctx.load_scene(sc, prof)
    W = H = size
    cam = S.room_camera(W, H)
    out = torch.zeros((H, W, 4), dtype=torch.float32, device=dev)
    ctx.render(cam, W, H, out, 0, max(1, warmup), stream)
    torch.cuda.synchronize()
    st = ctx.check_status(stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.render(cam, W, H, out, 1000, frames, stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / frames
    stats = ctx.render_stats()
    counters = ctx.render_counters()
    host = torch.empty((H, W, 4), dtype=torch.float32).pin_memory()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    for f in range(frames):
        ctx.render(cam, W, H, out, 2000 + f, 1, stream)
        host.copy_(out, non_blocking=True)
    f1.record(stream)
    torch.cuda.synchronize()
    ms_e2e = f0.elapsed_time(f1) / frames
    res = {"workload": "procedural room 1.04 M triangles, %dx%d paths/frame, max depth 8, HWSS 4 + spectral MIS, NEE + MIS, RR, "
                       "manifold NEE (2 occluders, 60 iterations, threshold 5e-5)" % (W, H),
           "status": int(st), "frames": frames, "ms_per_frame": ms, "paths_per_s": W * H / (ms * 1e-3),
           "e2e": {"paths_per_s": W * H / (ms_e2e * 1e-3), "d2h_bytes_per_frame": W * H * 16, "h2d_bytes_per_frame": 0},
           "rays_per_s": (stats["bounces"] + stats["shadow_rays"]) / (ms * 1e-3),
           # traversal's algorithmic bytes per frame (64 per node visit + 48 per triangle test,
           # counted by the kernels) over the frame time, against measured HBM bandwidth; the BVH
           # (38 MB nodes + 50 MB triangles) is mostly L2-resident, so this is a bound, not a limit
           "roofline": {"bound": "hbm", "achieved": counters["traversal_bytes"] / (ms * 1e-3) / 1e9,
                        "peak": peaks()[0]["hbm_gbs"], "unit": "GB/s",
                        "frac": counters["traversal_bytes"] / (ms * 1e-3) / 1e9 / peaks()[0]["hbm_gbs"],
                        "traversal_bytes_per_frame": counters["traversal_bytes"], "kind": "traversal over the whole frame"},
           "bounces_per_path": stats["bounces"] / (W * H), "shadow_rays_per_path": stats["shadow_rays"] / (W * H),
           "bsdf_evals_per_path": stats["bsdf_evals"] / (W * H), "gpu_launches_per_frame": 8 + 1 + 2 + 1}
    ctx.close()
    if cpu_seconds > 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        opt = capi_options(opts)
        w = h = 256
        ccam = S.room_camera(w, h)
        setups = []
        for _ in range(2):   # set-up alone (scene copy, BVH, light table): a 1-pixel render
            t0 = time.perf_counter()
            oracle.render(sc, prof, ccam, opt, 1, 1, frame=0)
            setups.append(time.perf_counter() - t0)
        setup = min(setups)
        calls, frames, t0 = 0, 2, time.perf_counter()
        while calls == 0 or time.perf_counter() - t0 < cpu_seconds + calls * setup:
            oracle.render(sc, prof, ccam, opt, w, h, frame=calls * frames, frames=frames)
            calls += 1
        dt = max(1e-6, time.perf_counter() - t0 - calls * setup)
        res["cpu_baseline"] = {"value": calls * frames * w * h / dt, "unit": "paths/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": "%d frames of a 256x256 image of the same view and options, %.1f s of rendering "
                                         "(per-call set-up of %.2f s excluded)" % (calls * frames, dt, setup)}
    return res


def relmse(x, ref, eps=1e-2, trim=0.0):
    """Relative MSE of an image against a reference: mean over pixels of the channel mean of
    (x - ref)^2 / (ref^2 + eps).  With trim > 0 the largest `trim` fraction of the per-pixel terms is
    left out (the outlier-robust relMSE of the rendering literature, which reports error without the
    rare firefly pixels that dominate the plain mean at finite sample counts)."""
    import numpy as np
    e = np.mean((x - ref) ** 2 / (ref ** 2 + eps), axis=-1).ravel()
    if trim > 0.0:
        k = int(len(e) * trim)
        if k > 0:
            e = np.partition(e, len(e) - k - 1)[:len(e) - k]
    return float(np.mean(e))


def learned_bench(dev, stream, prob=0.25, width=256, ref_spp=4096, budget_s=12.0, batch_spp=32):
    """Learned proposal against the analytic tracer on the 1.04 M-triangle procedural room (the render
    leg's scene and options at width^2), measured against an independent reference: the analytic
    tracer at ref_spp samples per pixel (frames disjoint from the compared renders).  The proposal
    is trained on 2^24 samples drawn from the exact samplers of the scene's materials (256 Adam steps
    x 65536, lr 1e-3).  Each tracer then renders batches of batch_spp frames for budget_s seconds
    (CUDA events), the running mean compared with the reference after every batch: relMSE (eps 1e-2)
    and the same with the 0.1 % largest per-pixel terms left out (trimmed relMSE).

    Reported: both convergence curves (spp, seconds, relMSE, trimmed relMSE); on the trimmed relMSE,
    the directly measured time each tracer needs to reach the lowest error both reach (training time
    included for the learned one) and their ratio; the curves fitted as V / spp + R (R the
    reference's own contribution: it is itself an analytic render, at ref_spp spp, and dominates
    these curves, so V is unstable and no time is projected from it); and the headline time to relMSE
    1e-3, from the variance per spp (each batch against the pooled mean of every render, see below),
    which needs no converged reference.  The plain relMSE is dominated by rare caustic and grazing-grating fireflies (single
    pixels 10^3 x the reference), so it does not fall as 1/spp within the budget and no fit is made
    on it."""
    import numpy as np
    import torch
    from pltfalcor_gb300 import scene as S, spectra
    from pltfalcor_gb300.bsdf import PLTContext
    prof, _ = spectra.standard_profiles()
    sc = S.procedural_scene()
    base = {"max_bounces": 8, "hwss": 4, "do_mnee": 1, "mnee_max_occluders": 2, "mnee_max_iterations": 60,
            "mnee_solver_threshold": 5e-5}
    W = H = width
    cam = S.room_camera(W, H)
    out = torch.zeros((H, W, 4), dtype=torch.float32, device=dev)

    def curve(ctx, ref, frame0, batches):
        acc = np.zeros((H, W, 3))
        spp, t_ms, pts = 0, 0.0, []
        ctx.render(cam, W, H, out, 1 << 26, 1, stream)     # warm-up (graph recording)
        torch.cuda.synchronize()
        while t_ms < budget_s * 1e3:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.render(cam, W, H, out, frame0 + spp, batch_spp, stream)
            e1.record(stream)
            torch.cuda.synchronize()
            t_ms += e0.elapsed_time(e1)
            img = out[..., :3].double().cpu().numpy()
            batches.append(img)
            acc += img * batch_spp
            spp += batch_spp
            pts.append((spp, t_ms * 1e-3, relmse(acc / spp, ref), relmse(acc / spp, ref, trim=1e-3)))
        return pts, acc / spp

    ctx = PLTContext(base)
    ctx.load_scene(sc, prof)
    ctx.render(cam, W, H, out, 1 << 28, ref_spp, stream)
    torch.cuda.synchronize()
    ref = out[..., :3].double().cpu().numpy()
    batches_p, batches_l = [], []
    plain, img_p = curve(ctx, ref, 0, batches_p)
    ctx.close()
    ctx = PLTContext(dict(base, learned_proposal=1, learned_proposal_prob=prob))
    ctx.load_scene(sc, prof)
    ctx.proposal_init(3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = ctx.proposal_train(256, batch=65536, lr=1e-3, seed=1)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    learned, img_l = curve(ctx, ref, 0, batches_l)
    st = ctx.check_status(stream)
    ctx.close()

    # fit relMSE(spp) = V / spp + R by least squares over the second half of each curve, with R shared
    # (the reference's error, equal for both comparisons in expectation)
    def design(pts):
        p = pts[len(pts) // 2:]
        return np.array([1.0 / s for s, _, _, _ in p]), np.array([m for _, _, _, m in p])
    xp, yp = design(plain)
    xl, yl = design(learned)
    A = np.zeros((len(xp) + len(xl), 3))
    A[:len(xp), 0], A[len(xp):, 1], A[:, 2] = xp, xl, 1.0
    (Vp, Vl, R), *_ = np.linalg.lstsq(A, np.concatenate([yp, yl]), rcond=None)
    ms_p = plain[-1][1] / plain[-1][0] * 1e3
    ms_l = learned[-1][1] / learned[-1][0] * 1e3
    # directly measured: first time each curve reaches the lowest trimmed relMSE both curves reach
    level = max(min(m for _, _, _, m in plain), min(m for _, _, _, m in learned))
    first = lambda pts, extra: next(t for _, t, _, m in pts if m <= level) + extra
    tm_p, tm_l = first(plain, 0.0), first(learned, train_s)
    # variance per spp without a converged reference: every batch of batch_spp frames is an
    # independent estimate of the same image from either tracer (both are unbiased), so each batch's
    # trimmed relMSE is taken against the pooled mean of all batches of both tracers and of the
    # reference render (~100x the spp of one batch, so its own error is negligible); the median over
    # a tracer's batches is its error at batch_spp, which falls as 1/spp.
    pooled = (sum(batches_p) + sum(batches_l)) * batch_spp + ref * ref_spp
    pooled /= (len(batches_p) + len(batches_l)) * batch_spp + ref_spp
    e_p = float(np.median([relmse(b, pooled, trim=1e-3) for b in batches_p]))
    e_l = float(np.median([relmse(b, pooled, trim=1e-3) for b in batches_l]))
    tv_p = e_p * batch_spp / 1e-3 * ms_p * 1e-3
    tv_l = e_l * batch_spp / 1e-3 * ms_l * 1e-3 + train_s
    curve = lambda pts: [[s, round(t, 4), round(m, 6), round(mt, 6)] for s, t, m, mt in pts[::max(1, len(pts) // 12)]] + \
        [[pts[-1][0], round(pts[-1][1], 4), round(pts[-1][2], 6), round(pts[-1][3], 6)]]
    return {"workload": "procedural room 1.04 M triangles, %dx%d, max depth 8, HWSS 4 + spectral MIS, NEE + MIS + manifold NEE, "
                        "RR; learned proposal probability %.2f, trained on 2^24 exact-sampler samples" % (W, H, prob),
            "reference": "analytic tracer, %d spp, frames disjoint from the compared renders" % ref_spp,
            "status": int(st), "budget_s_per_tracer": budget_s, "batch_spp": batch_spp,
            "curve_columns": ["spp", "seconds", "relmse", "relmse_trimmed_0.1%"],
            "curve_plain": curve(plain), "curve_learned": curve(learned),
            "image_mean_plain": float(img_p.mean()), "image_mean_learned": float(img_l.mean()), "image_mean_reference": float(ref.mean()),
            "ms_per_spp_plain": ms_p, "ms_per_spp_learned": ms_l, "train_s": train_s,
            "train_loss_first_last": [float(hist[:8].mean()), float(hist[-8:].mean())],
            "measured_equal_relmse": {"metric": "relmse_trimmed_0.1%", "relmse": level, "time_plain_s": tm_p, "time_learned_s": tm_l,
                                      "speedup": tm_p / tm_l},
            "fit": {"metric": "relmse_trimmed_0.1%", "V_plain": float(Vp), "V_learned": float(Vl), "R_reference": float(R),
                    "note": "V / spp + R over the second half of each curve; R (the reference's own error) dominates, so V is "
                            "unstable from run to run and no time is projected from it"},
            "variance_per_spp": {"metric": "relmse_trimmed_0.1%% of one %d-spp batch against the pooled mean of all renders, median "
                                           "over batches" % batch_spp,
                                 "relmse_plain": e_p, "relmse_learned": e_l, "batches_plain": len(batches_p), "batches_learned": len(batches_l),
                                 "time_to_relmse_1e-3_plain_s": tv_p, "time_to_relmse_1e-3_learned_s": tv_l},
            "time_to_relmse_1e-3_plain_s": tv_p, "time_to_relmse_1e-3_learned_s": tv_l, "speedup": tv_p / tv_l}


def scene_set_bench(dev, stream, count=64, frames=2):
    """Heterogeneous batched render: `count` seeded procedural rooms of uneven size (10 K-500 K
    triangles, 4 K-1 M primary rays each, log-uniform; every room with its own materials over the
    eight PLT types, gratings and up to 32-layer stacks included), HWSS 8, max depth 8, manifold
    NEE, learned proposal on (probability 0.25, trained on 2^24 exact-sampler samples).  Batched:
    all views in one plt_render_scenes wavefront per frame, replayed as a recorded CUDA graph, launch
    shape from plt_render_tune.  Against: the same views as `count` separate plt_render_scenes calls
    of one view each, launched directly (PLT_OPTION_NO_GRAPH) with the default launch shape.  Rays
    = closest-hit segments + shadow and manifold rays (the render statistics)."""
    import torch
    from pltfalcor_gb300 import capi, scene as S, spectra
    from pltfalcor_gb300.bsdf import PLTContext
    prof, _ = spectra.standard_profiles()
    t0 = time.perf_counter()
    rooms = S.scene_set(seed=4, count=count)
    gen_s = time.perf_counter() - t0
    recs, offs = S.merged_materials([r for r, _, _ in rooms])
    base = {"max_bounces": 8, "hwss": 8, "do_mnee": 1, "mnee_max_occluders": 2, "mnee_max_iterations": 60,
            "mnee_solver_threshold": 5e-5, "learned_proposal": 1, "learned_proposal_prob": 0.25}

    def context(flags):
        ctx = PLTContext(dict(base, flags=flags))
        ctx.set_spectral_profiles(prof)
        ctx.set_materials(recs)
        for (r, _, _), o in zip(rooms, offs):
            ctx.add_scene(r, o)
        ctx.proposal_init(3)
        ctx.proposal_train(256, batch=65536, lr=1e-3, seed=1)
        return ctx

    outs = [torch.zeros((h, w, 4), dtype=torch.float32, device=dev) for _, w, h in rooms]
    views = [(i, S.room_camera(w, h), w, h, o) for i, ((_, w, h), o) in enumerate(zip(rooms, outs))]
    paths = sum(w * h for _, w, h in rooms)
    t0 = time.perf_counter()
    ctx = context(0)
    ctx.render_scenes(views, 0, 1, stream)      # scene upload, light tables, buffers
    torch.cuda.synchronize()
    load_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    shape, tuned_ms = ctx.render_tune(views, 100, 1, stream)
    tune_s = time.perf_counter() - t0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.render_scenes(views, 1000, frames, stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_batched = e0.elapsed_time(e1) / frames
    st = ctx.check_status(stream)
    stats = ctx.render_stats()
    rays = stats["bounces"] + stats["shadow_rays"]
    ctx.close()
    ctx = context(capi.OPTION_NO_GRAPH)
    for v in views:
        ctx.render_scenes([v], 0, 1, stream)
    torch.cuda.synchronize()
    e0.record(stream)
    for v in views:
        ctx.render_scenes([v], 1000, frames, stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms_separate = e0.elapsed_time(e1) / frames
    ctx.close()
    tris = [r.n_tris for r, _, _ in rooms]
    return {"workload": "%d procedural rooms, %d-%d triangles (%d total), %d-%d primary rays (%d total), HWSS 8, depth 8, "
                        "manifold NEE, learned proposal on" % (count, min(tris), max(tris), sum(tris), min(w * h for _, w, h in rooms),
                                                               max(w * h for _, w, h in rooms), paths),
            "status": int(st), "frames": frames, "paths_per_frame": paths,
            "ms_per_frame_batched": ms_batched, "ms_per_frame_separate": ms_separate, "speedup": ms_separate / ms_batched,
            "paths_per_s_batched": paths / (ms_batched * 1e-3), "rays_per_s_batched": rays / (ms_batched * 1e-3),
            "rays_per_frame": int(rays), "launch_shape": shape, "tuned_ms_per_frame": tuned_ms,
            "scene_gen_s": gen_s, "load_s": load_s, "tune_s": tune_s}


def config0_bench(dev, stream, steps=200, cpu_seconds=0.0):
    """The reference's CPU-runnable case: the rough-dielectric eval + pdf batch, 65,536 queries,
    seed 0 (wi, wo uniform on the upper hemisphere, IOR 1.5 with Cauchy B = 0.0042 um^2,
    roughness 0.01-0.5, coherence area 5-50 um^2, unpolarised).  Inputs and outputs (5 MB) stay in
    L2 between launches.  Roofline: 80 algorithmic bytes per query and the oracle-counted FP32 and
    SFU operations (profiles/op_counts_rough_dielectric.json) against nominal rates at the clock."""
    import torch
    from pltfalcor_gb300 import capi, spectra
    from pltfalcor_gb300 import workloads as W
    from pltfalcor_gb300.bsdf import DeviceBatch, PLTContext
    prof, _ = spectra.standard_profiles()
    wl = W.rough_dielectric_batch(n=65536, seed=0, profiles=prof)
    ctx = PLTContext()
    ctx.set_spectral_profiles(prof)
    ctx.set_materials(wl.records)
    b = DeviceBatch(wl, device=dev)
    ops = capi.OP_EVAL | capi.OP_PDF
    q, r = b.queries(), b.results(ops)
    for _ in range(10):
        ctx.batch(q, r, ops, stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        ctx.batch(q, r, ops, stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    st = ctx.check_status(stream)
    ctx.close()
    qps = wl.n / (ms * 1e-3)
    out = {"workload": "rough_dielectric_batch: 65,536 eval+pdf queries, HWSS 1, seed 0", "status": int(st), "steps": steps,
           "ms_per_batch": ms, "queries_per_s": qps, "algorithmic_bytes_per_query": 80,
           "achieved_gbs": 80 * qps / 1e9}
    pk, _ = peaks()
    out["hbm_frac"] = out["achieved_gbs"] / pk["hbm_gbs"]
    ops_path = os.path.join(ROOT, "profiles", "op_counts_rough_dielectric.json")
    if os.path.exists(ops_path):
        with open(ops_path) as f:
            oc = json.load(f)
        mhz = pk.get("sm_max_mhz", 2070.0)
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        fp32_peak, sfu_peak = sms * 128 * 2 * mhz * 1e6 / 1e12, sms * 16 * mhz * 1e6 / 1e12
        out["fp32_frac"] = oc["mean_fp_per_query"] * qps / 1e12 / fp32_peak
        out["sfu_frac"] = oc["mean_sfu_per_query"] * qps / 1e12 / sfu_peak
    if cpu_seconds > 0:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        oracle.run(wl, ops=ops, threads=os.cpu_count())
        done, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < cpu_seconds:
            oracle.run(wl, ops=ops, threads=os.cpu_count())
            done += wl.n
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": done / dt, "unit": "queries/s", "cores": os.cpu_count(), "kind": "port",
                               "sample": "%d queries (the whole batch, repeated) in %.1f s, FP32 oracle, OpenMP" % (done, dt)}
    return out


def capi_options(overrides):
    import ctypes as C
    from pltfalcor_gb300 import capi
    o = capi.Options()
    capi.load_library().plt_options_default(C.byref(o))
    for k, v in overrides.items():
        setattr(o, k, v)
    return o


def run_reference(args):
    """The reference arm: the CPU restatement of the reference's BSDF code (the oracle; the reference
    path itself is Slang shader code with no CPU build and no graphics stack here) on all host
    threads, over the same batch as the GPU arm: each step is one pass over all args.n queries.
    Nothing here loads the product library: the spectral profiles come from the oracle's own
    profile builder."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from pltfalcor_gb300 import workloads as W
    threads = os.cpu_count()
    prof, _ = oracle.standard_profiles()
    wl = W.mixed_material_batch(n=args.n, profiles=prof)
    res = oracle.alloc_results(wl.n, wl.hwss)
    for _ in range(args.warmup):
        oracle.run(wl, threads=threads, res=res)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.run(wl, threads=threads, res=res)
    dt = time.perf_counter() - t0
    v = wl.n * args.steps / dt
    line = {"metric": METRIC, "value": v, "unit": "queries/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD, "queries_per_gpu": wl.n, "hwss": 1, "materials": int(len(wl.records)),
                       "step": "one pass over the whole batch"},
            "cpu_baseline": {"value": v, "unit": "queries/s", "cores": threads, "kind": "port",
                             "sample": "%d passes over the %d-query mixed-material batch, FP32 oracle restating the reference Slang "
                                       "BSDFs (the reference path is shader code with no CPU build), OpenMP" % (args.steps, wl.n)},
            "e2e": {"value": v, "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_ours(args):
    import torch
    import torch.distributed as dist
    from pltfalcor_gb300 import capi, spectra
    from pltfalcor_gb300 import workloads as W
    from pltfalcor_gb300.bsdf import DeviceBatch, PLTContext, _ptr

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)

    prof, _ = spectra.standard_profiles()
    wl = W.mixed_material_batch(n=args.n, seed=1 + rank, profiles=prof)
    ctx = PLTContext()
    ctx.set_spectral_profiles(prof)
    ctx.set_materials(wl.records)
    b = DeviceBatch(wl, device=dev)
    ops = capi.OP_EVAL | capi.OP_SAMPLE | capi.OP_PDF
    q, r = b.queries(), b.results(ops)

    sampler = ClockSampler(local if "CUDA_VISIBLE_DEVICES" not in os.environ else 0)
    sampler.start()
    for _ in range(args.warmup):
        ctx.batch(q, r, ops, stream)
    st = ctx.check_status(stream)
    if st != capi.PLT_OK:
        raise RuntimeError("device status %s" % capi.STATUS_NAMES[st])

    def barrier():
        if world > 1:
            dist.barrier()
    # per-kernel events: the library records them around its classify and shade launches
    kev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    for trio in kev:
        for ev in trio:
            ev.record(stream)              # creates the event so its handle can be passed down
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for trio in kev:
        ctx.lib.plt_set_timing_events(ctx.handle, *[C.c_void_p(ev.cuda_event) for ev in trio])
        ctx.batch(q, r, ops, stream)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ctx.lib.plt_set_timing_events(ctx.handle, None, None, None)
    ms = e0.elapsed_time(e1)
    classify_ms = sum(a.elapsed_time(b) for a, b, _ in kev) / args.steps
    shade_ms = sum(b.elapsed_time(c) for _, b, c in kev) / args.steps
    t = torch.tensor([ms], device=dev)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms_max = float(t.item())
    value = args.n * world * args.steps / (ms_max * 1e-3)

    # end to end through the C ABI with host buffers: plt_bsdf_batch_host on pinned host queries and
    # results (every step copies all inputs to the device and all requested outputs back, chunked
    # so copies in both directions overlap the kernels)
    # two sets of pinned host buffers: consecutive steps are independent batches submitted on two
    # alternating streams, so one call's input copies overlap the previous call's output copies
    # (each call is still ordered after the earlier work on its own stream)
    hbs = [DeviceBatch(wl, device="cpu", pin=True) for _ in range(2)]
    hqr = [(h.queries(), h.results(ops)) for h in hbs]
    hb = hbs[0]
    streams = [stream, torch.cuda.Stream(dev)]
    h_in = [hb.material, hb.v, hb.w, hb.lobe, hb.wavelengths, hb.stokes, hb.coherence]
    d_out = [b.out_stokes, b.out_coherence, b.out_pdf, b.out_sample_wo, b.out_sample_pdf, b.out_sample_weight,
             b.out_sample_lobe, b.out_sample_valid]
    h2d = sum(x.numel() * x.element_size() for x in h_in)
    d2h = sum(x.numel() * x.element_size() for x in d_out)

    def e2e_step(k):
        hq, hr = hqr[k % 2]
        ctx.batch_host(hq, hr, ops, streams[k % 2])
    for k in range(max(2, args.warmup)):
        e2e_step(k)
    torch.cuda.synchronize()
    barrier()
    f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    f0.record(stream)
    streams[1].wait_event(f0)
    for k in range(args.steps):
        e2e_step(k)
    done_b = torch.cuda.Event()
    done_b.record(streams[1])
    stream.wait_event(done_b)
    f1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms_e2e = f0.elapsed_time(f1)
    t = torch.tensor([ms_e2e], device=dev)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    e2e_value = args.n * world * args.steps / (float(t.item()) * 1e-3)
    clocks = sampler.stop()
    st = ctx.check_status(stream)
    if st != capi.PLT_OK:
        raise RuntimeError("device status %s" % capi.STATUS_NAMES[st])

    if rank == 0:
        pk, pk_kind = peaks()
        # dominant kernel: the shade kernel, timed by the events the library recorded around it
        launch_s = shade_ms * 1e-3
        bytes_per_launch = h2d + d2h
        achieved = bytes_per_launch / launch_s / 1e9
        roof = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / pk["hbm_gbs"], "traffic": None, "peak_kind": pk_kind,
                "kernel": "pltdev::bsdfShadeKernel<1>", "kernel_ms": shade_ms, "classify_kernel_ms": classify_ms,
                "algorithmic_bytes_per_launch": bytes_per_launch, "algorithmic_bytes_per_query": bytes_per_launch / args.n}
        prof_path = os.path.join(ROOT, "profiles", "bsdf_shade_mixed_material_4M.json")
        if os.path.exists(prof_path):
            with open(prof_path) as f:
                pj = json.load(f)
            if pj.get("dram_bytes_per_launch"):
                # per-launch DRAM bytes of one ncu capture, scaled by queries if this run's batch differs
                roof["traffic"] = pj["dram_bytes_per_launch"] * args.n / pj.get("queries_per_launch", args.n)
        ops_path = os.path.join(ROOT, "profiles", "op_counts_mixed_material.json")
        if os.path.exists(ops_path):
            with open(ops_path) as f:
                oc = json.load(f)
            mhz = (clocks or {}).get("sm_mhz") or pk.get("sm_max_mhz", 2070.0)
            sms = torch.cuda.get_device_properties(dev).multi_processor_count
            fp32_peak = sms * 128 * 2 * mhz * 1e6 / 1e12          # FMA lanes x 2 flops, nominal at the sampled clock
            sfu_peak = sms * 16 * mhz * 1e6 / 1e12                 # MUFU ops per clock per SM
            fp_q, sfu_q = oc["mean_fp_per_query"], oc["mean_sfu_per_query"]
            qps = args.n / launch_s
            roof["compute"] = {"fp32_tflops": fp_q * qps / 1e12, "fp32_peak_tflops_nominal": fp32_peak,
                               "fp32_frac": fp_q * qps / 1e12 / fp32_peak, "sfu_tops": sfu_q * qps / 1e12,
                               "sfu_peak_tops_nominal": sfu_peak, "sfu_frac": sfu_q * qps / 1e12 / sfu_peak,
                               "fp_ops_per_query": fp_q, "sfu_ops_per_query": sfu_q, "div_per_query": oc.get("mean_div_per_query")}
        line = {"metric": METRIC, "value": value, "unit": "queries/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": WORKLOAD, "queries_per_gpu": args.n, "hwss": 1, "materials": int(len(wl.records)),
                           "l2": "inputs %d MB + outputs %d MB per step exceed the 126 MB L2; no flush" % (h2d >> 20, d2h >> 20),
                           "parallelism": "independent shards per GPU" if world > 1 else "1 GPU"},
                "e2e": {"value": e2e_value, "unit": "queries/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                        "how": "plt_bsdf_batch_host on pinned host buffers, every input copied in and every output copied back "
                               "each step; independent steps on two alternating streams with two buffer sets"},
                "gpu_launches": 2 * args.steps, "roofline": roof, "clocks": clocks}
        line["config0"] = config0_bench(dev, stream, cpu_seconds=0.0 if (world > 1 or args.no_cpu_baseline) else 3.0)
        if not args.no_trace:
            line["trace"] = trace_bench(ctx, dev, stream, max(3, min(args.steps, 50)), max(1, args.warmup))
        if not args.no_render:
            line["render"] = render_bench(dev, stream, max(3, min(args.steps // 10, 16)), 1,
                                          cpu_seconds=0.0 if (world > 1 or args.no_cpu_baseline) else min(args.cpu_seconds, 10.0),
                                          size=args.render_size)
        if not args.no_learned:
            line["learned"] = learned_bench(dev, stream)
        if not args.no_scene_set:
            line["scene_set"] = scene_set_bench(dev, stream)
        if world == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(seconds=args.cpu_seconds)
        print(json.dumps(line))
    ctx.close()
    if world > 1:
        dist.destroy_process_group()


def per_material_bench(n, steps, warmup):
    """The BSDF shade kernel per material: the mixed-material batch of n queries, then each of its
    material types' queries alone (contiguous, n / 8 each), eval + sample + pdf at HWSS 1; CUDA events
    around the shade launch (plt_set_timing_events), median of `steps` after `warmup` untimed runs.
    With --steps 1 --warmup 0 the process launches exactly 9 shade kernels in that order (the
    profiling command of the per-material instruction mix).  Prints one JSON line."""
    import ctypes as C
    import numpy as np
    import torch
    from pltfalcor_gb300 import capi, spectra, workloads as W, materials as M
    from pltfalcor_gb300.bsdf import DeviceBatch, PLTContext
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    prof, _ = spectra.standard_profiles()
    full = W.mixed_material_batch(n=n, profiles=prof)
    ops = capi.OP_EVAL | capi.OP_SAMPLE | capi.OP_PDF
    ctx = PLTContext()
    ctx.set_spectral_profiles(prof)
    ctx.set_materials(full.records)
    s = torch.cuda.current_stream()

    def timed(wl):
        b = DeviceBatch(wl)
        q, r = b.queries(), b.results(ops)
        for _ in range(warmup):
            ctx.batch(q, r, ops, s)
        ms = []
        for _ in range(steps):
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            for e in ev:
                e.record(s)   # creates the events (torch creates them lazily); the library re-records them
            ctx.lib.plt_set_timing_events(ctx.handle, *[C.c_void_p(e.cuda_event) for e in ev])
            ctx.batch(q, r, ops, s)
            torch.cuda.synchronize()
            ms.append(ev[1].elapsed_time(ev[2]))
        ctx.lib.plt_set_timing_events(ctx.handle, None, None, None)
        assert ctx.check_status(s) == 0
        m = float(np.median(ms))
        return {"queries": wl.n, "shade_ms": m, "queries_per_s": wl.n / (m * 1e-3)}

    out = {"metric": "BSDF shade kernel per material (eval+sample+pdf, HWSS 1)", "mixed": timed(full)}
    types = full.meta["types"]
    for t, ty in enumerate(M.BENCH_TYPES):
        out[M.TYPE_NAMES[int(ty)]] = timed(full.subset(np.nonzero(types == t)[0]))
    out["sum_of_materials_ms"] = sum(v["shade_ms"] for k, v in out.items() if isinstance(v, dict) and k != "mixed")
    ctx.close()
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-trace", action="store_true")
    ap.add_argument("--no-render", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-scene-set", action="store_true")
    ap.add_argument("--render-size", type=int, default=1024, help="render leg image width = height (profiling uses small sizes)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--per-material", action="store_true", help="only the shade kernel per material (diagnostic), one JSON line")
    args = ap.parse_args()
    if args.per_material:
        per_material_bench(args.n, args.steps, args.warmup)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
