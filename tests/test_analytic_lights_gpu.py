"""Analytic lights in plt_render against the oracle's render: every light type (point / spot and
directional, whose zero-pdf samples the reference rejects; distant, rect, disc and sphere) together
with the environment map and emissive geometry, so light-type selection runs over three types;
and the rect light against the same quad as emissive geometry on the GPU.  Tolerances are written
in the tests."""
import ctypes as C

import numpy as np
import pytest

from pltfalcor_gb300 import capi
from pltfalcor_gb300 import scene as S

pytestmark = pytest.mark.gpu

MIN_IDENTICAL_PATHS = 0.97
PIXEL_RTOL = 2e-3
MIN_PIXEL_SHARE = 0.98
RECT = [[0.5, 0, 0, 0], [0, 0.5, 0, 0], [0, 0, -1, 6.0]]


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    return torch


def _options(**kw):
    o = capi.Options()
    capi.load_library().plt_options_default(C.byref(o))
    o.max_bounces, o.hwss = 6, 4
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def _lights():
    return [S.point_light((0.0, 0.0, 5.0), 8), S.directional_light((0.2, 0.1, -1.0), 8),
            S.distant_light((0.3, -0.4, -1.0), 8, half_angle=0.05),
            S.area_light("rect", [[0.8, 0, 0, -3.0], [0, 0.4, 0, 2.0], [0, 0, -1, 7.0]], 8),
            S.area_light("disc", [[0.6, 0, 0, 3.0], [0, 0.6, 0, -1.0], [0, 0, -1, 6.5]], 8),
            S.area_light("sphere", [[0.3, 0, 0, 2.0], [0, 0.3, 0, 3.0], [0, 0, 0.3, 4.0]], 8)]


def _render(torch, scene, prof, opt, cam, w, h, env=None, lights=None, frame=0, frames=1):
    from pltfalcor_gb300.bsdf import PLTContext
    ctx = PLTContext({f[0]: getattr(opt, f[0]) for f in capi.Options._fields_})
    ctx.load_scene(scene, prof)
    if env is not None:
        ctx.set_env_map(env["rgb"], env["intensity"], env["tint"], env["rotation"])
    if lights:
        ctx.set_analytic_lights(lights)
    out = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    ctx.render(cam, w, h, out, frame_begin=frame, frame_count=frames)
    torch.cuda.synchronize()
    st = ctx.check_status()
    recs = ctx.render_bounces(w * h, opt.max_bounces)
    ctx.close()
    assert st == capi.PLT_OK, capi.STATUS_NAMES.get(st, st)
    return out.cpu().numpy(), recs


@pytest.mark.parametrize("kw,with_env", [({}, True), ({"do_mnee": 0}, False), ({"hwss": 1}, True), ({"do_mis": 0}, False)])
def test_analytic_lights_match_oracle(torch_cuda, oracle_lib, product_lib, profiles, kw, with_env):
    import oracle
    prof = profiles[0]
    scene = S.open_scene(emitter=True)
    w, h = 48, 32
    cam = S.look_at_camera((0.0, -9.0, -3.0), (0.0, 0.0, 0.5), (0.0, 0.0, 1.0), 80.0, w / h)
    env = dict(rgb=S.sky_env(sun_radiance=5.0), intensity=0.5, tint=(1.0, 1.0, 1.0), rotation=(90.0, 0.0, 0.0)) if with_env else None
    opt = _options(**kw)
    gpu, grecs = _render(torch_cuda, scene, prof, opt, cam, w, h, env, _lights(), frame=4)
    orc, orecs, _ = oracle.render(scene, prof, cam, opt, w, h, frame=4, records=True, env=env, lights=_lights())
    assert np.isfinite(gpu).all()
    g = gpu[..., :3].reshape(-1, 3).astype(np.float64)
    o = orc.reshape(-1, 3).astype(np.float64)
    same = np.ones(len(g), bool)
    for a, b in zip(grecs, orecs):
        same &= (a == b).all(axis=1)
    scale = max(np.abs(o).mean(), 1e-6)
    rel = np.abs(g - o).max(axis=1) / np.maximum(np.abs(o).max(axis=1), 1e-3 * scale)
    ok = rel[same] <= PIXEL_RTOL
    msg = "%s env %s: identical paths %.4f, pixels within %.0e %.4f, mean g %.5g o %.5g" % (
        kw, with_env, same.mean(), PIXEL_RTOL, ok.mean(), g.mean(), o.mean())
    print(msg)
    assert same.mean() >= MIN_IDENTICAL_PATHS, msg
    assert ok.mean() >= MIN_PIXEL_SHARE, msg
    assert abs(g.mean() - o.mean()) <= 0.05 * abs(o.mean()) + 1e-6, msg


def test_rect_light_equals_emissive_quad(torch_cuda, product_lib, profiles):
    prof = profiles[0]
    w, h = 64, 48
    cam = S.look_at_camera((0.0, -9.0, 5.0), (0.0, 0.0, 0.5), (0.0, 0.0, 1.0), 70.0, w / h)
    opt = _options(max_bounces=0, do_mis=0, do_mnee=0, do_importance_sample_emitters=0)
    em, recs = _render(torch_cuda, S.floor_spheres_scene(emitter=True), prof, opt, cam, w, h, frames=128)
    an, _ = _render(torch_cuda, S.floor_spheres_scene(emitter=False), prof, opt, cam, w, h, lights=[S.area_light("rect", RECT, 8)],
                    frames=128)
    keep = ~np.isin(recs[0][:, 0], S.floor_spheres_scene(emitter=True).emissive_tris).reshape(h, w)
    a, b = an[..., :3][keep].mean(), em[..., :3][keep].mean()
    print("rect light %.5g, emissive quad %.5g" % (a, b))
    assert a > 0 and abs(a / b - 1) < 0.01


def test_analytic_light_api(torch_cuda, product_lib, profiles):
    from pltfalcor_gb300.bsdf import PLTContext
    lib = capi.load_library()
    ctx = PLTContext(None)
    ctx.set_spectral_profiles(profiles[0])
    bad = S.point_light((0, 0, 0), 8)
    bad.type = 9
    assert lib.plt_set_analytic_lights(ctx.handle, C.byref(bad), 1) == capi.PLT_INVALID_ARG
    bad = S.point_light((0, 0, 0), 10_000)
    assert lib.plt_set_analytic_lights(ctx.handle, C.byref(bad), 1) == capi.PLT_INVALID_ARG
    sing = S.area_light("rect", [[0, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]], 8)   # singular transform
    assert lib.plt_set_analytic_lights(ctx.handle, C.byref(sing), 1) == capi.PLT_INVALID_ARG
    ctx.set_analytic_lights(_lights())
    ctx.set_analytic_lights([])
    ctx.close()
