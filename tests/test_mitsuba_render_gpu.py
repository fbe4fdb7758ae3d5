"""A Mitsuba 3 scene imported by pltfalcor_gb300/mitsuba.py (every mapped BSDF type, an RGB area
emitter, a constant environment, a point light) rendered by plt_render against the oracle's render
of the same import."""
import ctypes as C

import numpy as np
import pytest

import mitsuba_fixture
from pltfalcor_gb300 import capi, mitsuba

pytestmark = pytest.mark.gpu


def test_mitsuba_scene_renders_like_oracle(product_lib, oracle_lib, tmp_path):
    torch = pytest.importorskip("torch")
    import oracle
    from pltfalcor_gb300.bsdf import PLTContext
    sc, prof, cam, w, h, lights, env = mitsuba.build(mitsuba.load(str(mitsuba_fixture.write(tmp_path))))
    opt = capi.Options()
    capi.load_library().plt_options_default(C.byref(opt))
    opt.max_bounces, opt.hwss = 6, 4
    ctx = PLTContext({f[0]: getattr(opt, f[0]) for f in capi.Options._fields_})
    ctx.load_scene(sc, prof)
    ctx.set_env_map(env["rgb"], env["intensity"])
    ctx.set_analytic_lights(lights)
    out = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    ctx.render(cam, w, h, out, 0, 1)
    torch.cuda.synchronize()
    assert ctx.check_status() == capi.PLT_OK
    grecs = ctx.render_bounces(w * h, opt.max_bounces)
    ctx.close()
    orc, orecs, _ = oracle.render(sc, prof, cam, opt, w, h, records=True, env=dict(rgb=env["rgb"], intensity=env["intensity"]),
                                  lights=lights)
    g = out.cpu().numpy()[..., :3]
    assert np.isfinite(g).all() and g.mean() > 0
    same = np.ones(w * h, bool)
    for a, b in zip(grecs, orecs):
        same &= (a == b).all(axis=1)
    print("identical paths %.4f, mean g %.5g o %.5g" % (same.mean(), g.mean(), orc.mean()))
    assert same.mean() >= 0.97
    assert abs(g.mean() - orc.mean()) <= 0.05 * abs(orc.mean())
