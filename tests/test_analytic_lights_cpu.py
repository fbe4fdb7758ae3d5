"""Analytic lights in the oracle's render (CPU): the reference's zero-pdf rejection of point and
directional light samples, and a rect area light against the same quad as emissive geometry
(same spectrum, NEE at the primary hit only)."""
import ctypes as C

import numpy as np
import pytest

from pltfalcor_gb300 import capi
from pltfalcor_gb300 import scene as S


@pytest.fixture(scope="module")
def orc(oracle_lib):
    import oracle
    return oracle


def _options(**kw):
    o = capi.Options()
    capi.load_library().plt_options_default(C.byref(o))
    o.max_bounces, o.hwss = 0, 4
    for k, v in kw.items():
        setattr(o, k, v)
    return o


CAM = dict(pos=(0.0, -9.0, 5.0), target=(0.0, 0.0, 0.5))
RECT = [[0.5, 0, 0, 0], [0, 0.5, 0, 0], [0, 0, -1, 6.0]]    # the emissive quad of floor_spheres_scene, facing down


def _cam(w, h):
    return S.look_at_camera(CAM["pos"], CAM["target"], (0.0, 0.0, 1.0), 70.0, w / h)


def test_point_and_directional_lights_contribute_nothing(orc, profiles):
    w, h = 24, 16
    sc = S.floor_spheres_scene(emitter=False)
    lights = [S.point_light((0.0, 0.0, 5.0), 8), S.point_light((1.0, 0.0, 4.0), 8, (0, 0, -1), 0.5, 0.1),
              S.directional_light((0.2, 0.1, -1.0), 8)]
    img = orc.render(sc, profiles[0], _cam(w, h), _options(max_bounces=3), w, h, frames=2, lights=lights)
    assert (img == 0).all()


def test_rect_light_equals_emissive_quad(orc, profiles):
    """Direct light at the primary hit from a rect light and from the same quad as emissive geometry
    agree (the emissive quad also multiplies by rgbToSpectrum(white) <= 1 and uses snorm16 normals);
    pixels whose primary ray hits the emissive quad are left out."""
    w, h = 32, 24
    prof = profiles[0]
    kw = dict(do_mis=0, do_mnee=0, do_importance_sample_emitters=0)
    em_img, recs, _ = orc.render(S.floor_spheres_scene(emitter=True), prof, _cam(w, h), _options(**kw), w, h, frames=64, records=True)
    an_img = orc.render(S.floor_spheres_scene(emitter=False), prof, _cam(w, h), _options(**kw), w, h, frames=64,
                        lights=[S.area_light("rect", RECT, 8)])
    sc = S.floor_spheres_scene(emitter=True)
    keep = ~np.isin(recs[0][:, 0], sc.emissive_tris).reshape(h, w)
    a, b = an_img[keep].mean(), em_img[keep].mean()
    assert a > 0
    assert abs(a / b - 1) < 0.02, (a, b)
