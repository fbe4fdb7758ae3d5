"""Scene sets: several independent scenes rendered by one plt_render_scenes call (one wavefront over
all views' paths) against each scene rendered alone by plt_render.

Each view's paths seed the generator with view-local pixel coordinates, traverse their own scene's
BVH (a root in the combined node array) and sample their own scene's lights, so a batched view must
reproduce the separate render.  The only difference allowed is the summation order of deferred
manifold-walk contributions (double-precision atomics), hence the tolerance below.
"""
import ctypes as C

import numpy as np
import pytest

from pltfalcor_gb300 import capi
from pltfalcor_gb300 import scene as S

pytestmark = pytest.mark.gpu

RTOL, ATOL = 1e-5, 1e-5


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    return torch


@pytest.fixture(scope="module")
def rooms():
    return [S.procedural_scene(seed=11, n_spheres=6, sphere_level=2, n_quads=30, box_subdiv=4),
            S.procedural_scene(seed=12, n_spheres=2, sphere_level=3, n_quads=10, box_subdiv=6),
            S.procedural_scene(seed=13, n_spheres=10, sphere_level=1, n_quads=50, box_subdiv=3)]


OPTS = {"max_bounces": 6, "hwss": 4, "do_mnee": 1}


def _separate(torch, room, prof, cam, w, h, frame, frames, opts, params=None):
    from pltfalcor_gb300.bsdf import PLTContext
    ctx = PLTContext(opts)
    ctx.load_scene(room, prof)
    if params is not None:
        ctx.proposal_set_params(params)
    out = torch.zeros((h, w, 4), dtype=torch.float32, device="cuda")
    ctx.render(cam, w, h, out, frame, frames)
    torch.cuda.synchronize()
    assert ctx.check_status() == capi.PLT_OK
    ctx.close()
    return out.cpu().numpy()


def _batched(torch, rooms, prof, views, frame, frames, opts, params=None):
    from pltfalcor_gb300.bsdf import PLTContext
    ctx = PLTContext(opts)
    recs, offs = S.merged_materials(rooms)
    ctx.set_spectral_profiles(prof)
    ctx.set_materials(recs)
    ids = [ctx.add_scene(r, o) for r, o in zip(rooms, offs)]
    assert ids == list(range(len(rooms)))
    if params is not None:
        ctx.proposal_set_params(params)
    outs = [torch.zeros((h, w, 4), dtype=torch.float32, device="cuda") for (_, _, w, h) in views]
    ctx.render_scenes([(sid, cam, w, h, o) for (sid, cam, w, h), o in zip(views, outs)], frame, frames)
    torch.cuda.synchronize()
    assert ctx.check_status() == capi.PLT_OK
    stats = ctx.render_stats()
    ctx.close()
    return [o.cpu().numpy() for o in outs], stats


def _views():
    near = S.look_at_camera((2.0, -8.0, 0.0), (0.0, 0.0, 3.0), (0.0, 0.0, 1.0), 60.0, 1.0)
    return [(0, S.room_camera(48, 32), 48, 32), (1, S.room_camera(40, 40), 40, 40), (2, S.room_camera(32, 24), 32, 24),
            (0, near, 24, 24)]


def test_scene_set_equals_separate_renders(torch_cuda, product_lib, profiles, rooms):
    prof = profiles[0]
    views = _views()
    batched, stats = _batched(torch_cuda, rooms, prof, views, 5, 2, OPTS)
    assert stats["paths"] == sum(w * h for _, _, w, h in views)
    for (sid, cam, w, h), b in zip(views, batched):
        ref = _separate(torch_cuda, rooms[sid], prof, cam, w, h, 5, 2, OPTS)
        assert np.isfinite(b).all()
        np.testing.assert_allclose(b, ref, rtol=RTOL, atol=ATOL * max(1.0, np.abs(ref).mean()))


def test_scene_set_learned_equals_separate(torch_cuda, product_lib, profiles, rooms):
    from pltfalcor_gb300.bsdf import PLTContext
    prof = profiles[0]
    opts = dict(OPTS, learned_proposal=1, learned_proposal_prob=0.5)
    seed_ctx = PLTContext(opts)
    seed_ctx.set_spectral_profiles(prof)
    seed_ctx.set_materials(rooms[0].records)
    seed_ctx.proposal_init(21)
    params = seed_ctx.proposal_params()
    seed_ctx.close()
    views = _views()[:2]
    batched, _ = _batched(torch_cuda, rooms, prof, views, 0, 1, opts, params)
    for (sid, cam, w, h), b in zip(views, batched):
        ref = _separate(torch_cuda, rooms[sid], prof, cam, w, h, 0, 1, opts, params)
        np.testing.assert_allclose(b, ref, rtol=RTOL, atol=ATOL * max(1.0, np.abs(ref).mean()))


def test_scene_set_rejects_bad_views(torch_cuda, product_lib, profiles, rooms):
    from pltfalcor_gb300.bsdf import PLTContext
    lib = capi.load_library()
    ctx = PLTContext(OPTS)
    recs, offs = S.merged_materials(rooms[:1])
    ctx.set_spectral_profiles(profiles[0])
    ctx.set_materials(recs)
    ctx.add_scene(rooms[0], offs[0])
    out = torch_cuda.zeros((8, 8, 4), dtype=torch_cuda.float32, device="cuda")
    v = (capi.RenderView * 1)()
    v[0].scene, v[0].width, v[0].height = 1, 8, 8        # no scene 1
    v[0].camera = S.room_camera(8, 8)
    v[0].out_rgba = out.data_ptr()
    assert lib.plt_render_scenes(ctx.handle, v, 1, 0, 1, None) == capi.PLT_INVALID_ARG
    v[0].scene = 0
    v[0].out_rgba = out.data_ptr() + 4                   # misaligned output
    assert lib.plt_render_scenes(ctx.handle, v, 1, 0, 1, None) == capi.PLT_INVALID_ARG
    d = capi.SceneDesc()
    assert lib.plt_add_scene(ctx.handle, C.byref(d), None) == capi.PLT_INVALID_ARG
    ctx.clear_scenes()
    v[0].out_rgba = out.data_ptr()
    assert lib.plt_render_scenes(ctx.handle, v, 1, 0, 1, None) == capi.PLT_INVALID_ARG
    ctx.close()


def _render_set(torch, rooms, prof, views, frame, frames, opts, shape=None, tune=False):
    from pltfalcor_gb300.bsdf import PLTContext
    ctx = PLTContext(opts)
    recs, offs = S.merged_materials(rooms)
    ctx.set_spectral_profiles(prof)
    ctx.set_materials(recs)
    for r, o in zip(rooms, offs):
        ctx.add_scene(r, o)
    if opts.get("learned_proposal"):
        ctx.proposal_init(5)
    if shape is not None:
        ctx.set_launch_shape(*shape)
    outs = [torch.zeros((h, w, 4), dtype=torch.float32, device="cuda") for (_, _, w, h) in views]
    vv = [(sid, cam, w, h, o) for (sid, cam, w, h), o in zip(views, outs)]
    tuned = ctx.render_tune(vv, 1000, 1) if tune else None
    ctx.render_scenes(vv, frame, frames)
    torch.cuda.synchronize()
    assert ctx.check_status() == capi.PLT_OK
    ctx.close()
    return [o.cpu().numpy() for o in outs], tuned


@pytest.mark.parametrize("learned", [0, 1])
def test_waves_graphs_and_shapes_do_not_change_results(torch_cuda, product_lib, profiles, rooms, learned):
    """Waves of 700 paths, small grids, direct launches instead of the recorded frame graph, and the
    autotuner's choice all give the default render's image."""
    prof = profiles[0]
    views = _views()
    opts = dict(OPTS, learned_proposal=learned, learned_proposal_prob=0.5)
    ref, _ = _render_set(torch_cuda, rooms, prof, views, 2, 2, opts)
    variants = [dict(shape=(700, 1, 1, 1, 2)), dict(shape=(0, 2, 1, 2, 1)), dict(shape=(0, 0, 0, 0, 2)), dict(tune=True)]
    nograph = dict(opts, flags=capi.OPTION_NO_GRAPH)
    outs = [_render_set(torch_cuda, rooms, prof, views, 2, 2, opts, **v) for v in variants]
    outs.append(_render_set(torch_cuda, rooms, prof, views, 2, 2, nograph))
    for (imgs, tuned) in outs:
        if tuned is not None:
            print("tuned shape", tuned)
        for a, b in zip(imgs, ref):
            np.testing.assert_allclose(a, b, rtol=RTOL, atol=ATOL * max(1.0, np.abs(b).mean()))
