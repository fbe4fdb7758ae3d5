"""Render parity against the oracle on the scene the render benchmark times, and on a batched
HWSS-8 scene set.

1. The procedural room of the render benchmark (1.04 M triangles: the closed box, 200 level-4
   icospheres, 500 random quads, the D65 area light and the glass sphere for manifold NEE) with the
   benchmark's options (max depth 8, HWSS 4 with spectral MIS, NEE + MIS, manifold NEE with 2
   occluders and 60 iterations at threshold 5e-5, Russian roulette) at 96 x 96: one frame with its
   bounce records, then two frames accumulated at another frame index.
2. Three small rooms rendered together by plt_render_scenes (one wavefront over all views' paths)
   at HWSS 8, each view compared with the oracle's render of its own room alone.

The criteria are those of tests/test_render_gpu.py: identical bounce records on >= 97 % of paths,
>= 98 % of pixels on identical paths within 2e-3 relative, and image means within 5 %.
"""
import numpy as np
import pytest

from pltfalcor_gb300 import capi
from pltfalcor_gb300 import scene as S
from test_render_gpu import _compare, _options, _render_gpu

pytestmark = pytest.mark.gpu

BENCH_OPTS = {"max_bounces": 8, "hwss": 4, "do_mnee": 1, "mnee_max_occluders": 2, "mnee_max_iterations": 60,
              "mnee_solver_threshold": 5e-5}


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    return torch


@pytest.fixture(scope="module")
def bench_room():
    return S.procedural_scene()


def test_bench_scene_matches_oracle(torch_cuda, oracle_lib, product_lib, profiles, bench_room):
    import oracle
    prof = profiles[0]
    assert bench_room.n_tris > 1_000_000
    w = h = 96
    cam = S.room_camera(w, h)
    opt = _options(**BENCH_OPTS)
    gpu, grecs, stats = _render_gpu(torch_cuda, bench_room, prof, opt, cam, w, h, frame=0)
    orc, orecs, ostats = oracle.render(bench_room, prof, cam, opt, w, h, frame=0, records=True)
    assert np.isfinite(gpu).all()
    same = _compare(gpu, orc, grecs, orecs, "bench room 96x96 frame 0")
    # the manifold walks run: paths through the glass sphere exist and reach the light
    assert stats["shadow_rays"] > w * h
    assert abs(stats["shadow_rays"] - int(ostats[1])) <= 0.05 * int(ostats[1]) + 10
    assert same.mean() >= 0.97


def test_bench_scene_frames_match_oracle(torch_cuda, oracle_lib, product_lib, profiles, bench_room):
    """Frames 5 and 6 each against the oracle (records of that frame), and their two-frame
    accumulation against the mean of the two single-frame renders."""
    import oracle
    prof = profiles[0]
    w = h = 64
    cam = S.room_camera(w, h)
    opt = _options(**BENCH_OPTS)
    singles = []
    for f in (5, 6):
        gpu, grecs, _ = _render_gpu(torch_cuda, bench_room, prof, opt, cam, w, h, frame=f)
        orc, orecs, _ = oracle.render(bench_room, prof, cam, opt, w, h, frame=f, records=True)
        _compare(gpu, orc, grecs, orecs, "bench room 64x64 frame %d" % f)
        singles.append(gpu[..., :3].astype(np.float64))
    both, _, _ = _render_gpu(torch_cuda, bench_room, prof, opt, cam, w, h, frame=5, frames=2)
    np.testing.assert_allclose(both[..., :3], 0.5 * (singles[0] + singles[1]), rtol=1e-5, atol=1e-6)


def test_scene_set_hwss8_matches_oracle(torch_cuda, oracle_lib, product_lib, profiles):
    import oracle
    from pltfalcor_gb300.bsdf import PLTContext
    prof = profiles[0]
    rooms = [S.procedural_scene(seed=11, n_spheres=6, sphere_level=2, n_quads=30, box_subdiv=4),
             S.procedural_scene(seed=12, n_spheres=2, sphere_level=3, n_quads=10, box_subdiv=6),
             S.procedural_scene(seed=13, n_spheres=10, sphere_level=1, n_quads=50, box_subdiv=3)]
    views = [(0, S.room_camera(48, 32), 48, 32), (1, S.room_camera(40, 40), 40, 40), (2, S.room_camera(32, 24), 32, 24)]
    kw = {"max_bounces": 8, "hwss": 8, "do_mnee": 1}
    opt = _options(**kw)
    fields = {f[0]: getattr(opt, f[0]) for f in capi.Options._fields_}
    ctx = PLTContext(fields)
    recs, offs = S.merged_materials(rooms)
    ctx.set_spectral_profiles(prof)
    ctx.set_materials(recs)
    for r, o in zip(rooms, offs):
        ctx.add_scene(r, o)
    outs = [torch_cuda.zeros((h, w, 4), dtype=torch_cuda.float32, device="cuda") for (_, _, w, h) in views]
    ctx.render_scenes([(sid, cam, w, h, o) for (sid, cam, w, h), o in zip(views, outs)], 3, 1)
    torch_cuda.cuda.synchronize()
    assert ctx.check_status() == capi.PLT_OK
    total = sum(w * h for (_, _, w, h) in views)
    grecs = ctx.render_bounces(total, opt.max_bounces)
    ctx.close()
    # the batched records hold triangle ids of the combined scene set: scene k's start after the
    # triangles of scenes 0..k-1
    tri_base = np.cumsum([0] + [r.n_tris for r in rooms])
    base = 0
    for (sid, cam, w, h), out in zip(views, outs):
        room = rooms[sid]
        orc, orecs, _ = oracle.render(room, prof, cam, opt, w, h, frame=3, records=True)
        prim = grecs[0][base:base + w * h]
        hit = prim < np.uint32(tri_base[-1])
        prim = np.where(hit, prim - np.uint32(tri_base[sid]), prim)
        view_recs = [prim] + [g[base:base + w * h] for g in grecs[1:]]
        _compare(out.cpu().numpy(), orc, view_recs, orecs, "scene set view %d (HWSS 8)" % sid)
        base += w * h
