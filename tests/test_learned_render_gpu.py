"""The learned MIS proposal inside plt_render (options.learned_proposal) on the small procedural room.

- parity: the GPU render with the proposal against the CPU oracle's restatement of the same sample
  pass (oracle/plt_oracle_pt.cpp, the network in double with the GPU's BF16 rounding), with the same
  network parameters.  The network's FP32 accumulation order differs from the oracle's, so a
  primary sample drawn from the mixture can move slightly; the bounds are looser than the analytic
  tracer's (written below);
- unbiasedness: the proposal draws the surface sampler's primary sample and divides the path weight
  by its one-sample MIS density, so the learned and the analytic tracer converge to the same image:
  image means agree within the Monte Carlo error estimated from independent batches of frames;
- gain: after training on the scene's materials, the per-pixel error at equal spp and the time per
  spp of both tracers are measured and printed (error ratio and time-to-equal-error ratio); the
  trained tracer's error must stay within a stated factor of the analytic tracer's.
"""
import time

import numpy as np
import pytest

from pltfalcor_gb300 import capi
from pltfalcor_gb300 import scene as S

pytestmark = pytest.mark.gpu

FLAG_LEARNED = 0x40
PROB = 0.5
# parity with the oracle: share of identical bounce records, per-pixel tolerance on identical paths
MIN_IDENTICAL_PATHS = 0.93
PIXEL_RTOL = 2e-2
MIN_PIXEL_SHARE = 0.95
# unbiasedness: |mean_learned - mean_plain| <= Z_BOUND standard errors
Z_BOUND = 4.0
# gain: trained learned relMSE at equal spp <= this factor times the analytic tracer's
MAX_ERROR_FACTOR = 1.5


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    return torch


@pytest.fixture(scope="module")
def room():
    return S.small_scene()


def _fields(**kw):
    lib = capi.load_library()
    import ctypes as C
    o = capi.Options()
    lib.plt_options_default(C.byref(o))
    o.max_bounces = 8
    o.hwss = 4
    for k, v in kw.items():
        setattr(o, k, v)
    return o, {f[0]: getattr(o, f[0]) for f in capi.Options._fields_}


def _context(room, prof, learned, params=None, train_steps=0, **kw):
    from pltfalcor_gb300.bsdf import PLTContext
    opt, fields = _fields(learned_proposal=1 if learned else 0, learned_proposal_prob=PROB, **kw)
    ctx = PLTContext(fields)
    ctx.load_scene(room, prof)
    if learned:
        if params is not None:
            ctx.proposal_set_params(params)
        else:
            ctx.proposal_init(11)
        if train_steps:
            ctx.proposal_train(train_steps, batch=65536, lr=1e-3, seed=5)
    return ctx, opt


def _render(torch, ctx, cam, w, h, frame, frames):
    out = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    ctx.render(cam, w, h, out, frame_begin=frame, frame_count=frames)
    torch.cuda.synchronize()
    assert ctx.check_status() == capi.PLT_OK
    return out[..., :3].double().cpu().numpy()


def test_learned_render_matches_oracle(torch_cuda, oracle_lib, product_lib, profiles, room):
    import oracle
    prof = profiles[0]
    w, h = 64, 48
    cam = S.room_camera(w, h)
    ctx, opt = _context(room, prof, True, train_steps=16)
    params = ctx.proposal_params()
    gpu = _render(torch_cuda, ctx, cam, w, h, 0, 1)
    grecs = ctx.render_bounces(w * h, opt.max_bounces)
    ctx.close()
    orc, orecs, _ = oracle.render(room, prof, cam, opt, w, h, frame=0, records=True, proposal_params=params)
    g = gpu.reshape(-1, 3)
    o = orc.reshape(-1, 3).astype(np.float64)
    same = np.ones(len(g), bool)
    for a, b in zip(grecs, orecs):
        same &= (a == b).all(axis=1)
    learned_vertices = (orecs[2] & FLAG_LEARNED) != 0
    scale = max(np.abs(o).mean(), 1e-6)
    rel = np.abs(g - o).max(axis=1) / np.maximum(np.abs(o).max(axis=1), 1e-3 * scale)
    ok = rel[same] <= PIXEL_RTOL
    msg = "learned parity: identical paths %.4f, proposal vertices %d, pixels within %.0e %.4f, mean g %.5g o %.5g" % (
        same.mean(), learned_vertices.sum(), PIXEL_RTOL, ok.mean(), g.mean(), o.mean())
    print(msg)
    assert learned_vertices.sum() > 0.2 * (orecs[0] != 0xFFFFFFFF).sum(), msg
    assert same.mean() >= MIN_IDENTICAL_PATHS, msg
    assert ok.mean() >= MIN_PIXEL_SHARE, msg
    assert abs(g.mean() - o.mean()) <= 0.05 * abs(o.mean()), msg


def _batches(torch, ctx, cam, w, h, frame0, nb, per):
    return np.stack([_render(torch, ctx, cam, w, h, frame0 + i * per, per) for i in range(nb)])


def test_learned_render_unbiased(torch_cuda, product_lib, profiles, room):
    prof = profiles[0]
    w, h = 64, 48
    cam = S.room_camera(w, h)
    nb, per = 16, 32
    plain, _ = _context(room, prof, False)
    a = _batches(torch_cuda, plain, cam, w, h, 0, nb, per)
    plain.close()
    learned, _ = _context(room, prof, True, train_steps=64)
    b = _batches(torch_cuda, learned, cam, w, h, 100000, nb, per)
    learned.close()
    ma, mb = a.mean(axis=(1, 2, 3)), b.mean(axis=(1, 2, 3))      # image mean of each batch
    se = np.sqrt(ma.var(ddof=1) / nb + mb.var(ddof=1) / nb)
    z = abs(mb.mean() - ma.mean()) / se
    print("unbiased: plain %.5g learned %.5g (se %.3g, z %.2f)" % (ma.mean(), mb.mean(), se, z))
    assert np.isfinite(b).all()
    assert z <= Z_BOUND


def test_learned_gain_reported(torch_cuda, product_lib, profiles, room):
    """Trained proposal against the analytic tracer at equal spp: per-batch relMSE against the mean of
    both tracers' batches (both are unbiased for the same image), its median over the batches, the
    time per spp, and the resulting time-to-equal-error ratio (relMSE falls as 1/spp)."""
    prof = profiles[0]
    w, h = 64, 48
    cam = S.room_camera(w, h)
    spp, reps = 16, 16

    def measure(ctx):
        imgs, times = [], []
        _render(torch_cuda, ctx, cam, w, h, 1 << 20, 1)
        for r in range(reps):
            t0 = time.perf_counter()
            imgs.append(_render(torch_cuda, ctx, cam, w, h, r * spp, spp))
            times.append(time.perf_counter() - t0)
        return np.stack(imgs), float(np.median(times))

    plain, _ = _context(room, prof, False)
    a, t_plain = measure(plain)
    plain.close()
    learned, _ = _context(room, prof, True, train_steps=256)
    b, t_learned = measure(learned)
    learned.close()
    ref = 0.5 * (a.mean(0) + b.mean(0))
    rel = lambda x: np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2), axis=(1, 2, 3))
    e_plain, e_learned = float(np.median(rel(a))), float(np.median(rel(b)))
    speedup = (e_plain * t_plain) / (e_learned * t_learned)
    print("gain: median relMSE at %d spp plain %.4g learned %.4g (ratio %.3f); time per %d spp plain %.4f s learned %.4f s; "
          "time-to-equal-error speed-up %.3f" % (spp, e_plain, e_learned, e_plain / e_learned, spp, t_plain, t_learned, speedup))
    assert np.isfinite(b).all()
    assert e_learned <= MAX_ERROR_FACTOR * e_plain
