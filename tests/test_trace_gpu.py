"""BVH traversal on the GPU vs the brute-force CPU oracle (same watertight test): closest-hit
primitive, distance and barycentrics bit-exact; occlusion bit-exact; edge cases."""
import numpy as np
import pytest

import oracle
from pltfalcor_gb300 import capi
from pltfalcor_gb300 import scene as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    return torch


@pytest.fixture(scope="module")
def ctx(torch_cuda, product_lib):
    from pltfalcor_gb300.bsdf import PLTContext
    c = PLTContext()
    yield c
    c.close()


def gpu_closest(ctx, torch, o, d, tmin=None, tmax=None):
    dev = torch.device("cuda")
    to = lambda a: None if a is None else torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev)
    go, gd, g0, g1 = to(o), to(d), to(tmin), to(tmax)
    n = len(o) // 3
    prim = torch.zeros(n, dtype=torch.int32, device=dev)
    t = torch.zeros(n, dtype=torch.float32, device=dev)
    bary = torch.zeros(2 * n, dtype=torch.float32, device=dev)
    stats = torch.zeros(2, dtype=torch.int64, device=dev)
    r = ctx.rays(go, gd, g0, g1, stats)
    ctx.trace_closest(r, prim, t, bary)
    assert ctx.check_status() == capi.PLT_OK
    return prim.cpu().numpy().view(np.uint32), t.cpu().numpy(), bary.cpu().numpy(), stats.cpu().numpy()


def gpu_any(ctx, torch, o, d, tmin=None, tmax=None):
    dev = torch.device("cuda")
    to = lambda a: None if a is None else torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev)
    n = len(o) // 3
    occ = torch.zeros(n, dtype=torch.int32, device=dev)
    ctx.trace_any(ctx.rays(to(o), to(d), to(tmin), to(tmax)), occ)
    assert ctx.check_status() == capi.PLT_OK
    return occ.cpu().numpy().view(np.uint32)


def assert_bitexact(g, o):
    gp, gt, gb, _ = g
    op, ot, ob = o
    assert np.array_equal(gp, op), "prim mismatch on %d rays" % int((gp != op).sum())
    assert np.array_equal(gt.view(np.uint32), ot.view(np.uint32))
    assert np.array_equal(gb.view(np.uint32), ob.view(np.uint32))


def test_closest_hit_small_scene(ctx, torch_cuda):
    sc = S.procedural_scene(n_spheres=20, sphere_level=2, n_quads=50, box_subdiv=8)
    ctx.set_scene(sc.vertices, sc.indices, sc.tri_material)
    st = ctx.scene_stats()
    assert st["triangles"] == sc.n_tris and st["nodes"] > 0
    tv = sc.triangle_vertices()
    o, d = S.random_rays(65536, 5, sc.bounds, tv)
    g = gpu_closest(ctx, torch_cuda, o, d)
    assert_bitexact(g, oracle.trace_brute(tv, o, d))
    assert g[3][0] > 0 and g[3][1] > 0  # traversal counters ran


def test_closest_hit_ray_intervals(ctx, torch_cuda):
    sc = S.procedural_scene(n_spheres=12, sphere_level=3, n_quads=40, box_subdiv=4, seed=9)
    ctx.set_scene(sc.vertices, sc.indices, sc.tri_material)
    tv = sc.triangle_vertices()
    o, d = S.random_rays(32768, 6, sc.bounds, tv)
    rng = np.random.default_rng(3)
    tmin = (rng.random(32768) * 2.0).astype(np.float32)
    tmax = (tmin + rng.random(32768) * 8.0).astype(np.float32)
    tmax[:100] = tmin[:100]          # zero-length intervals
    tmin[100:200] = tmax[100:200] + 1  # empty intervals
    assert_bitexact(gpu_closest(ctx, torch_cuda, o, d, tmin, tmax), oracle.trace_brute(tv, o, d, tmin, tmax))
    occ_g = gpu_any(ctx, torch_cuda, o, d, tmin, tmax)
    occ_o = oracle.trace_brute(tv, o, d, tmin, tmax, any_hit=True)
    assert np.array_equal(occ_g, occ_o)
    assert 0.05 < occ_g.mean() < 0.95


def test_full_size_scene_subset(ctx, torch_cuda):
    """The ~1.04 M-triangle path-tracing scene, a brute-force-checkable subset of rays."""
    sc = S.procedural_scene()
    ctx.set_scene(sc.vertices, sc.indices, sc.tri_material)
    tv = sc.triangle_vertices()
    o, d = S.random_rays(384, 11, sc.bounds, tv)
    assert_bitexact(gpu_closest(ctx, torch_cuda, o, d), oracle.trace_brute(tv, o, d))
    occ = gpu_any(ctx, torch_cuda, o, d, None, np.full(384, 3.0, np.float32))
    assert np.array_equal(occ, oracle.trace_brute(tv, o, d, None, np.full(384, 3.0, np.float32), any_hit=True))


def test_edge_cases(ctx, torch_cuda):
    o = np.zeros(9, np.float32)  # three rays from the origin along +x, +y, +z (SoA planes)
    d = np.float32([1, 0, 0,   # x components
                    0, 1, 0,   # y
                    0, 0, 1])  # z
    # empty scene: everything misses
    ctx.set_scene(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.uint32))
    p, t, _, _ = gpu_closest(ctx, torch_cuda, o, d)
    assert (p == 0xFFFFFFFF).all() and (t == -1).all()
    # one triangle crossing +x at distance 2, plus a degenerate (zero-area) triangle on the +y axis
    v = np.float32([[2, -1, -1], [2, 1, -1], [2, 0, 1], [0, 3, 0], [0, 3, 0], [0, 3, 0]])
    f = np.uint32([[0, 1, 2], [3, 4, 5]])
    ctx.set_scene(v, f)
    p, t, b, _ = gpu_closest(ctx, torch_cuda, o, d)
    tv = v[f].reshape(-1, 9)
    assert_bitexact((p, t, b, None), oracle.trace_brute(tv, o, d))
    assert p[0] == 0 and t[0] == 2.0 and p[1] == 0xFFFFFFFF
    with pytest.raises(capi.PLTError):
        ctx.set_scene(v, np.uint32([[0, 1, 9]]))
    with pytest.raises(capi.PLTError):
        bad = v.copy()
        bad[0, 0] = np.nan
        ctx.set_scene(bad, f)
