"""The environment light on the GPU: the sampler (plt_env_map_query) against the oracle's, and
plt_render of open scenes lit by the map (NEE light-type selection between the map and emissive
geometry, distant beams, manifold walks towards a distant light, onMiss with MIS) against the
oracle's render, plus a check that NEE and BSDF sampling estimate the same direct light.
Tolerances are written in the tests.
"""
import ctypes as C

import numpy as np
import pytest

from pltfalcor_gb300 import capi
from pltfalcor_gb300 import scene as S

pytestmark = pytest.mark.gpu

MIN_IDENTICAL_PATHS = 0.97
PIXEL_RTOL = 2e-3
MIN_PIXEL_SHARE = 0.98
ENV = dict(rgb=None, intensity=1.3, tint=(1.0, 0.9, 0.8), rotation=(90.0, 0.0, 25.0))


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    return torch


@pytest.fixture(scope="module")
def env():
    return dict(ENV, rgb=S.sky_env())


def _options(**kw):
    o = capi.Options()
    capi.load_library().plt_options_default(C.byref(o))
    o.max_bounces = 6
    o.hwss = 4
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def _ctx(opt):
    from pltfalcor_gb300.bsdf import PLTContext
    return PLTContext({f[0]: getattr(opt, f[0]) for f in capi.Options._fields_})


def _render(torch, scene, prof, opt, env, cam, w, h, frame=0, frames=1):
    ctx = _ctx(opt)
    ctx.load_scene(scene, prof)
    if env is not None:
        ctx.set_env_map(env["rgb"], env["intensity"], env["tint"], env["rotation"])
    out = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    ctx.render(cam, w, h, out, frame_begin=frame, frame_count=frames)
    torch.cuda.synchronize()
    st = ctx.check_status()
    recs = ctx.render_bounces(w * h, opt.max_bounces)
    ctx.close()
    assert st == capi.PLT_OK, capi.STATUS_NAMES.get(st, st)
    return out.cpu().numpy(), recs


def _camera(w, h):
    return S.look_at_camera((0.0, -9.0, -3.0), (0.0, 0.0, 0.5), (0.0, 0.0, 1.0), 80.0, w / h)


def test_sampler_matches_oracle(torch_cuda, oracle_lib, product_lib, env):
    import oracle
    n = 1 << 15
    rng = np.random.default_rng(11)
    u = rng.uniform(0, 1, (n, 2)).astype(np.float32)
    z = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    d = np.stack([np.sqrt(1 - z * z) * np.cos(ph), np.sqrt(1 - z * z) * np.sin(ph), z], -1).astype(np.float32)
    ctx = _ctx(_options())
    ctx.set_env_map(env["rgb"], env["intensity"], env["tint"], env["rotation"])
    g = ctx.env_map_query(torch_cuda.from_numpy(u).cuda(), torch_cuda.from_numpy(d).cuda()).cpu().numpy()
    ctx.close()
    o = oracle.env_query(env, u, d)
    # same texel choice: directions agree to FP32 transcendental accuracy, pdfs to the importance
    # map's summation rounding; a choice at a 2x2 split threshold may differ
    close = (np.abs(g[:, :3] - o[:, :3]).max(axis=1) < 1e-4) & np.isclose(g[:, 3], o[:, 3], rtol=1e-4)
    assert close.mean() > 0.999, close.mean()
    np.testing.assert_allclose(g[close, 4:7], o[close, 4:7], rtol=2e-3, atol=1e-4)
    # eval / evalPdf of the given directions
    same = np.isclose(g[:, 11], o[:, 11], rtol=1e-4)
    assert same.mean() > 0.999, same.mean()
    np.testing.assert_allclose(g[:, 8:11], o[:, 8:11], rtol=2e-3, atol=1e-4)


def test_env_api_rejects_bad_input(torch_cuda, product_lib):
    lib = capi.load_library()
    ctx = _ctx(_options())
    out = torch_cuda.zeros((4, 12), dtype=torch_cuda.float32, device="cuda")
    u = torch_cuda.zeros((4, 2), dtype=torch_cuda.float32, device="cuda")
    assert lib.plt_env_map_query(ctx.handle, C.c_void_p(u.data_ptr()), None, 4, C.c_void_p(out.data_ptr()), None) == capi.PLT_INVALID_ARG
    px = (C.c_float * 12)(*([1.0] * 12))
    assert lib.plt_set_env_map(ctx.handle, px, 2, 2, 2, 1.0, None, None) == capi.PLT_INVALID_ARG    # channels
    assert lib.plt_set_env_map(ctx.handle, px, 0, 2, 3, 1.0, None, None) == capi.PLT_INVALID_ARG    # empty
    assert lib.plt_set_env_map(ctx.handle, px, 2, 2, 3, -1.0, None, None) == capi.PLT_INVALID_ARG   # intensity
    bad = (C.c_float * 12)(*([1.0] * 11 + [float("nan")]))
    assert lib.plt_set_env_map(ctx.handle, bad, 2, 2, 3, 1.0, None, None) == capi.PLT_INVALID_ARG
    assert lib.plt_set_env_map(ctx.handle, px, 2, 2, 3, 1.0, None, None) == capi.PLT_OK
    assert lib.plt_env_map_query(ctx.handle, C.c_void_p(u.data_ptr()), None, 4, C.c_void_p(out.data_ptr()), None) == capi.PLT_OK
    torch_cuda.cuda.synchronize()
    np.testing.assert_allclose(out[:, 3].cpu().numpy(), 1 / (4 * np.pi), rtol=1e-5)
    assert lib.plt_clear_env_map(ctx.handle) == capi.PLT_OK
    assert lib.plt_env_map_query(ctx.handle, C.c_void_p(u.data_ptr()), None, 4, C.c_void_p(out.data_ptr()), None) == capi.PLT_INVALID_ARG
    ctx.close()


def _compare(gpu, orc, grecs, orecs, label):
    g = gpu[..., :3].reshape(-1, 3).astype(np.float64)
    o = orc.reshape(-1, 3).astype(np.float64)
    same = np.ones(len(g), bool)
    for a, b in zip(grecs, orecs):
        same &= (a == b).all(axis=1)
    scale = max(np.abs(o).mean(), 1e-6)
    rel = np.abs(g - o).max(axis=1) / np.maximum(np.abs(o).max(axis=1), 1e-3 * scale)
    ok = rel[same] <= PIXEL_RTOL
    msg = "%s: identical paths %.4f, pixels within %.0e %.4f (worst %.3g), mean g %.5g o %.5g" % (
        label, same.mean(), PIXEL_RTOL, ok.mean(), rel[same].max() if same.any() else 0, g.mean(), o.mean())
    print(msg)
    assert same.mean() >= MIN_IDENTICAL_PATHS, msg
    assert ok.mean() >= MIN_PIXEL_SHARE, msg
    assert abs(g.mean() - o.mean()) <= 0.05 * abs(o.mean()) + 1e-6, msg


@pytest.mark.parametrize("emitter,kw", [(True, {}), (False, {}), (True, {"do_mnee": 0}), (True, {"do_mis": 0}),
                                        (True, {"hwss": 1}), (False, {"hwss": 8, "nee_use_per_tile_sg": 1})])
def test_env_render_matches_oracle(torch_cuda, oracle_lib, product_lib, profiles, env, emitter, kw):
    import oracle
    prof = profiles[0]
    scene = S.open_scene(emitter=emitter)
    w, h = 48, 32
    cam = _camera(w, h)
    opt = _options(**kw)
    gpu, grecs = _render(torch_cuda, scene, prof, opt, env, cam, w, h, frame=2)
    orc, orecs, _ = oracle.render(scene, prof, cam, opt, w, h, frame=2, records=True, env=env)
    assert np.isfinite(gpu).all()
    _compare(gpu, orc, grecs, orecs, "emitter %s %s" % (emitter, kw))


def test_env_off_and_cleared(torch_cuda, product_lib, profiles, env):
    """use_env_light = 0 and a cleared map both render without the environment (the emitter only)."""
    prof = profiles[0]
    scene = S.open_scene()
    w, h = 32, 24
    cam = _camera(w, h)
    base, _ = _render(torch_cuda, scene, prof, _options(), None, cam, w, h)
    off, _ = _render(torch_cuda, scene, prof, _options(use_env_light=0), env, cam, w, h)
    np.testing.assert_array_equal(off, base)
    on, _ = _render(torch_cuda, scene, prof, _options(), env, cam, w, h)
    sky = base[..., :3].sum(-1) == 0          # mostly camera rays that escape: black without the map
    assert sky.mean() > 0.2
    assert (on[..., :3].sum(-1)[sky] > 0).mean() > 0.9
    assert on[..., :3].mean() > base[..., :3].mean()


@pytest.mark.parametrize("emitter", [False, True])
def test_env_direct_light_estimators_agree(torch_cuda, product_lib, profiles, env, emitter):
    """Direct light at the primary hit estimated by NEE (light-type selection between the map and
    the emitter, the map's importance sampler) and by BSDF sampling alone (the escaped or emitter-
    hitting ray from the primary hit, onMiss) converge to the same image mean.  Both paths end at
    the light (max_bounces 0 for NEE, 1 for BSDF sampling), where the bounce record's path
    contribution holds exactly the pdfs of the sampled directions before it; at vertices where a
    path continues, the reference's record also holds the next direction's pdf
    (pltpt_sample.rt.slang:122-128 appends after path.pdf *= bsdfSample.pdf), which NEE and
    emission there inherit, so longer paths are not compared this way.  The emitter's wavelengths
    are drawn uniformly (do_importance_sample_emitters = 0): its importance-sampled wavelengths come
    from the same generator stream as the primary hit's direction in the sample pass (both passes
    seed UniformSampleGenerator(pixel, frame)), which correlates the two on BSDF-sampled emitter hits."""
    prof = profiles[0]
    scene = S.floor_spheres_scene(emitter)
    w, h = 64, 48
    cam = S.look_at_camera((0.0, -9.0, 5.0), (0.0, 0.0, 0.5), (0.0, 0.0, 1.0), 70.0, w / h)
    envd = dict(env, rgb=S.sky_env(sun_radiance=5.0))
    kw = {"do_importance_sample_emitters": 0}
    a, _ = _render(torch_cuda, scene, prof, _options(max_bounces=0, do_mnee=0, do_mis=0, **kw), envd, cam, w, h, frames=128)
    b, _ = _render(torch_cuda, scene, prof, _options(max_bounces=1, do_nee=0, **kw), envd, cam, w, h, frames=1024)
    ma, mb = a[..., :3].mean(), b[..., :3].mean()
    print("emitter %s: NEE direct %.5g, BSDF-sampled direct %.5g" % (emitter, ma, mb))
    assert abs(ma / mb - 1) < 0.02
