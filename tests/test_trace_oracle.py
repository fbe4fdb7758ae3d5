"""CPU checks of the brute-force intersection oracle: watertightness of the reference's ray/triangle
test on closed meshes (rays from inside aimed exactly at shared vertices and edges never leak)
and hits at known distances."""
import numpy as np

import oracle
from pltfalcor_gb300 import scene as S


def test_watertight_closed_mesh(oracle_lib):
    v, f = S.icosphere(3)
    v = (v * 2.0 + np.array([0.3, -0.2, 0.1])).astype(np.float32)
    tv = np.ascontiguousarray(v[f].reshape(-1, 9))
    rng = np.random.default_rng(7)
    n = 20000
    origins = (np.array([0.3, -0.2, 0.1]) + 0.5 * (rng.random((n, 3)) - 0.5)).astype(np.float32)
    # targets: vertices and edge midpoints of random triangles
    pick = rng.integers(0, len(f), n)
    w = rng.integers(0, 6, n)
    tri = v[f[pick]].astype(np.float64)
    tgt = np.select([w[:, None] == k for k in range(5)],
                    [tri[:, 0], tri[:, 1], tri[:, 2], 0.5 * (tri[:, 0] + tri[:, 1]), 0.5 * (tri[:, 1] + tri[:, 2])],
                    0.5 * (tri[:, 2] + tri[:, 0]))
    d = (tgt - origins).astype(np.float32)
    prim, t, _ = oracle.trace_brute(tv, origins.T.reshape(-1), d.T.reshape(-1))
    assert (prim != 0xFFFFFFFF).all(), "ray leaked through a shared edge or vertex"
    assert (t > 0).all()


def test_known_distance_and_barycentrics(oracle_lib):
    tv = np.float32([[2, -1, -1, 2, 1, -1, 2, 0, 1]])
    o = np.float32([0, 0, 0])
    d = np.float32([1, 0, 0])
    prim, t, b = oracle.trace_brute(tv, o, d)
    assert prim[0] == 0 and t[0] == 2.0
    assert abs(b[0] - 0.25) < 1e-6 and abs(b[1] - 0.5) < 1e-6


def test_oracle_bvh_equals_brute_force(oracle_lib):
    """The path-tracing oracle casts rays through its own BVH; on the small room (random rays, a
    fifth aimed exactly at vertices and edge midpoints, plus zero and degenerate directions) it
    returns exactly the brute-force hits, distances and barycentrics, and the same occlusion."""
    sc = S.small_scene()
    tv = sc.triangle_vertices()
    o, d = S.random_rays(20000, 11, sc.bounds, tv)
    d = d.reshape(3, -1)
    d[:, :50] = 0.0                      # zero direction: no hit
    d[0, 50:100] = 0.0                   # axis-aligned components
    d = d.reshape(-1)
    tmax = np.full(20000, 3.0e38, np.float32)
    tmax[::7] = 2.5
    pb, tb, bb = oracle.trace_brute(tv, o, d, tmax=tmax)
    pv, tv2, bv = oracle.trace_brute(tv, o, d, tmax=tmax, bvh=True)
    assert (pb == pv).all()
    assert (pb[:50] == 0xFFFFFFFF).all()
    hit = pb != 0xFFFFFFFF
    assert (tb[hit] == tv2[hit]).all() and (bb.reshape(2, -1)[:, hit] == bv.reshape(2, -1)[:, hit]).all()
    ob = oracle.trace_brute(tv, o, d, tmax=tmax, any_hit=True)
    ov = oracle.trace_brute(tv, o, d, tmax=tmax, any_hit=True, bvh=True)
    assert (ob == ov).all()
