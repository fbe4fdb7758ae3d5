"""Mitsuba 3 import (pltfalcor_gb300/mitsuba.py): the reference importer's BSDF -> PLT material
mapping (IOR table and Abbe numbers, convertGSSigma2, named and spectral conductor IORs, nested
coated conductor, grating, twosided, unsupported types), shapes, area emitters, sensor and lights."""
import numpy as np

import mitsuba_fixture
from pltfalcor_gb300 import materials as M
from pltfalcor_gb300 import mitsuba


def _f16(bits):
    return float(np.asarray(bits, np.uint16).view(np.float16))


def test_helpers():
    assert mitsuba.lookup_ior("BK7") == (1.5046, 64.0)
    assert abs(mitsuba.convert_gs_sigma2(100.0) - 2.0 * (1.0 - 0.1 ** (1.0 / 32.0))) < 1e-12
    wl, v = mitsuba.rgb_to_spectrum_samples((1.0, 1.0, 1.0))
    assert len(wl) == 16 and wl[0] == 380.0 and wl[-1] == 720.0 and v[-1] == 0.0


def test_import_structure(product_lib, tmp_path):
    ms = mitsuba.load(str(mitsuba_fixture.write(tmp_path)))
    types = [int(r["type"][0]) for r in ms.records]
    assert types == [M.DIFFUSE, M.DIELECTRIC, M.CONDUCTOR, M.CONDUCTOR, M.COATED_CONDUCTOR, M.GRATED_CONDUCTOR, M.DIFFUSE,
                     M.THIN_DIELECTRIC, M.DIFFUSE, M.DIELECTRIC]
    floor, glass, gold, custom, coated, grating, emitter, film, plastic, water = [r[0] for r in ms.records]
    assert floor["flags"] & 1                                   # twosided
    assert abs(_f16(glass["ior"]) - 1.5046) < 1e-3 and abs(_f16(glass["specular"][0]) - 0.52 * 0.5046 / 64.0) < 2e-5
    assert abs(_f16(glass["specular"][3]) - 1.000277) < 1e-3     # ext_ior air
    assert _f16(water["specular"][0]) == 0.0                    # float IOR: infinite Abbe number
    assert abs(_f16(water["specular"][1]) - mitsuba.convert_gs_sigma2(100.0)) < 1e-3
    assert (gold["ior_n_spectral_id"], gold["ior_k_spectral_id"]) == (0, 1)
    assert (custom["ior_n_spectral_id"], custom["ior_k_spectral_id"]) == (10, 11)   # 9: the point light
    assert (coated["ior_n_spectral_id"], coated["ior_k_spectral_id"]) == (4, 5) and abs(_f16(coated["data1"][0]) - 20.0) < 1e-2
    assert (grating["ior_n_spectral_id"], int(grating["data1"][3]) & 0xFF) == (6, 4)
    assert emitter["emission_spectral_id"] == 12
    assert abs(_f16(plastic["base_color"][0]) - 1.0) < 1e-3 and _f16(plastic["base_color"][1]) == 0.0
    assert any("plastic" in w for w in ms.warnings)
    assert (ms.width, ms.height) == (48, 32) and ms.camera["fov"] == 60.0
    assert ms.env["rgb"].shape == (1, 1, 3) and len(ms.lights) == 1


def test_build(product_lib, tmp_path):
    sc, prof, cam, w, h, lights, env = mitsuba.build(mitsuba.load(str(mitsuba_fixture.write(tmp_path))))
    assert len(prof) == 13                                      # 9 standard + eta, k + emission + point light
    assert len(sc.emissive_tris) == 2
    # the emissive rectangle was turned over (rotate 180 about x) and faces the floor
    e = sc.emissive_tris[0]
    assert sc.normals[sc.indices[e][0]][2] < -0.99
    assert abs(lights[0].surface_area - 1.0) < 1e-6
    # 2 + 1280 + 12 + 1 + 2 + 64 + 2 + 2 + 2 + 2 triangles
    assert sc.n_tris == 2 + 1280 + 12 + 1 + 2 + 64 + 2 + 2 + 2 + 2
