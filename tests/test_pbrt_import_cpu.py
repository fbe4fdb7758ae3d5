"""PBRT-v4 import (pltfalcor_gb300/pbrt.py): the reference importer's PLT material mapping and its
roughness rule, shapes, transforms, camera, lights and warnings, on a scene written by the test."""
import numpy as np

import pbrt_fixture
from pltfalcor_gb300 import materials as M
from pltfalcor_gb300 import pbrt


def _f16(bits):
    return float(np.asarray(bits, np.uint16).view(np.float16))


def test_import_structure(product_lib, tmp_path):
    ps = pbrt.load(str(pbrt_fixture.write(tmp_path)))
    types = [int(r["type"][0]) for r in ps.records]
    assert types == [M.DIFFUSE, M.DIELECTRIC, M.COATED_OPAQUE_DIELECTRIC, M.CONDUCTOR, M.DIFFUSE]
    diel, coat, cond = ps.records[1][0], ps.records[2][0], ps.records[3][0]
    assert abs(_f16(diel["ior"]) - 1.33) < 1e-3
    assert abs(_f16(diel["specular"][1]) - 0.04) < 1e-4          # remaproughness false: u + v
    assert abs(_f16(diel["specular"][0]) - 0.0026) < 1e-5        # Cauchy B of Abbe 100 at IoR 1.5
    assert abs(_f16(coat["specular"][1]) - np.sqrt(0.2)) < 1e-3  # sqrt(u + v)
    assert (cond["ior_n_spectral_id"], cond["ior_k_spectral_id"]) == (4, 5)   # Cu in standard_profiles
    assert ps.camera["fov"] == 45.0 and (ps.width, ps.height) == (48, 32)
    assert len(ps.lights) == 1 and ps.lights[0][0] == "point" and ps.env["rgb"].shape[2] == 3
    assert any("area light" in w for w in ps.warnings) and any("measured" in w for w in ps.warnings)
    sc, prof, cam, w, h, lights, env = pbrt.build(ps)
    # 2 floor + 1280 sphere + 2 + 2 (quads) + 2 (bilinear) + 1
    assert sc.n_tris == 2 + 1280 + 4 + 2 + 1
    assert len(sc.emissive_tris) == 0 and len(prof) == 10 and len(lights) == 1
    # the binary PLY is the ascii one moved up by 2
    v = sc.vertices[sc.indices[1282:1286].ravel()]
    np.testing.assert_allclose(v[6:] - v[:6], np.tile([0.0, 0.0, 2.0], (6, 1)), atol=1e-6)


def test_area_lights_option(product_lib, tmp_path):
    ps = pbrt.load(str(pbrt_fixture.write(tmp_path)), area_lights=True)
    sc, prof, *_ = pbrt.build(ps)
    assert len(sc.emissive_tris) == 2 and len(prof) == 11
    assert int(sc.records["type"][sc.tri_material[sc.emissive_tris[0]]]) == M.DIFFUSE
