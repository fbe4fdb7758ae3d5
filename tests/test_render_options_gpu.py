"""PLTPT pass options beyond the light-transport switches, against the oracle
(PLTPT.cpp:147-175): sampleGenerator (TinyUniformSampleGenerator), alphaMasking with an alpha-0
material, and the debug views (debugView, debugViewIntensity; pltpt_debug.slangh,
pltpt_solve.rt.slang:102-106, 319-325, 449-475).

The criteria are those of tests/test_render_gpu.py: identical bounce records on >= 97 % of paths,
>= 98 % of pixels on identical paths within 2e-3 relative, image means within 5 %.
"""
import numpy as np
import pytest

from pltfalcor_gb300 import capi
from pltfalcor_gb300 import scene as S
from test_render_gpu import _compare, _options, _render_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    return torch


@pytest.fixture(scope="module")
def room():
    return S.small_scene()


def test_tiny_sample_generator(torch_cuda, oracle_lib, product_lib, profiles, room):
    import oracle
    w, h = 48, 32
    cam = S.room_camera(w, h)
    opt = _options(sample_generator=capi.SAMPLE_GENERATOR_TINY_UNIFORM)
    gpu, grecs, _ = _render_gpu(torch_cuda, room, profiles[0], opt, cam, w, h, frame=4)
    orc, orecs, _ = oracle.render(room, profiles[0], cam, opt, w, h, frame=4, records=True)
    _compare(gpu, orc, grecs, orecs, "tiny uniform generator")
    # a different generator draws different paths than the default one
    dflt, drecs, _ = _render_gpu(torch_cuda, room, profiles[0], _options(), cam, w, h, frame=4)
    assert not all(np.array_equal(a, b) for a, b in zip(grecs, drecs))


def _alpha_room(room):
    """The small room with one wall-and-quad material made fully transparent (alpha 0)."""
    import copy
    r = copy.copy(room)
    r.records = room.records.copy()
    counts = np.bincount(room.tri_material, minlength=len(room.records))
    counts[[room.light_material, room.mnee_material]] = 0
    m = int(np.argmax(counts))
    r.records["base_color"][m, 3] = 0   # binary16 zero
    return r, m


def test_alpha_masking(torch_cuda, oracle_lib, product_lib, profiles, room):
    import oracle
    r, m = _alpha_room(room)
    w, h = 48, 32
    cam = S.room_camera(w, h)
    imgs = []
    for am in (1, 0):
        opt = _options(alpha_masking=am)
        gpu, grecs, _ = _render_gpu(torch_cuda, r, profiles[0], opt, cam, w, h, frame=2)
        orc, orecs, _ = oracle.render(r, profiles[0], cam, opt, w, h, frame=2, records=True)
        _compare(gpu, orc, grecs, orecs, "alpha masking %d" % am)
        prims = grecs[0]
        hit = prims < np.uint32(r.n_tris)
        on_masked = np.isin(prims[hit], np.nonzero(r.tri_material == m)[0])
        # masked: no bounce record lies on the transparent material; unmasked: some do
        assert (on_masked.sum() == 0) == (am == 1)
        imgs.append(gpu)
    assert not np.allclose(imgs[0], imgs[1])


VIEWS = [capi.DEBUG_VIEW_NANS, capi.DEBUG_VIEW_INFS, capi.DEBUG_VIEW_PATH_LENGTH, capi.DEBUG_VIEW_HWSS_COMPS,
         capi.DEBUG_VIEW_NORMALS, capi.DEBUG_VIEW_UVS, capi.DEBUG_VIEW_COHERENCE_AREA, capi.DEBUG_VIEW_COHERENCE_ANISOTROPY,
         capi.DEBUG_VIEW_POLARIZATION, capi.DEBUG_VIEW_MNEE_ITERATIONS, capi.DEBUG_VIEW_MNEE_BOUNCES]


@pytest.mark.parametrize("view", VIEWS)
def test_debug_view_matches_oracle(torch_cuda, oracle_lib, product_lib, profiles, room, view):
    import oracle
    w, h = 48, 32
    cam = S.room_camera(w, h)
    opt = _options(debug_view=view, debug_view_intensity=1.0)
    gpu, grecs, _ = _render_gpu(torch_cuda, room, profiles[0], opt, cam, w, h, frame=1)
    orc, orecs, _ = oracle.render(room, profiles[0], cam, opt, w, h, frame=1, records=True)
    assert np.isfinite(gpu).all()
    if view in (capi.DEBUG_VIEW_NANS, capi.DEBUG_VIEW_INFS, capi.DEBUG_VIEW_UVS):
        # the path sums are finite by construction (only finite contributions are added), so these
        # views write nothing or black: the image is black at intensity 1
        assert np.abs(gpu[..., :3]).max() == 0.0 and np.abs(orc).max() == 0.0
        return
    assert np.abs(gpu[..., :3]).max() > 0.0
    if view == capi.DEBUG_VIEW_MNEE_BOUNCES:
        # a sparse image: only pixels whose manifold walk succeeded are lit, and a few walks are
        # ill-conditioned enough to succeed on one side only; compare the lit pixels
        lit_g, lit_o = (gpu[..., :3] != 0).any(axis=-1), (orc != 0).any(axis=-1)
        assert lit_o.sum() > 0
        assert (lit_g != lit_o).sum() <= max(3, 0.1 * lit_o.sum()), (lit_g.sum(), lit_o.sum())
        both = lit_g & lit_o
        np.testing.assert_allclose(gpu[..., :3][both], orc[both], rtol=2e-3, atol=1e-6)
        return
    _compare(gpu, orc, grecs, orecs, "debug view %d" % view)


def test_debug_view_intensity_blends(torch_cuda, product_lib, profiles, room):
    """debugViewIntensity t: colour + t (debug - colour), so t = 1/2 is the mean of t = 0 and t = 1."""
    w, h = 32, 24
    cam = S.room_camera(w, h)
    out = {}
    for t in (0.0, 0.5, 1.0):
        opt = _options(debug_view=capi.DEBUG_VIEW_PATH_LENGTH, debug_view_intensity=t)
        out[t] = _render_gpu(torch_cuda, room, profiles[0], opt, cam, w, h, frame=3)[0][..., :3].astype(np.float64)
    plain = _render_gpu(torch_cuda, room, profiles[0], _options(), cam, w, h, frame=3)[0][..., :3].astype(np.float64)
    # (a debug view runs the manifold walks inline: only the float summation order differs)
    np.testing.assert_allclose(out[0.0], plain, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(out[0.5], 0.5 * (out[0.0] + out[1.0]), rtol=1e-5, atol=1e-6)


def test_option_values_rejected(torch_cuda, product_lib):
    import ctypes as C
    lib = capi.load_library()
    for kw, want in (({"debug_view": 14}, capi.PLT_INVALID_ARG), ({"sample_generator": 2}, capi.PLT_INVALID_ARG),
                     ({"debug_view": capi.DEBUG_VIEW_ALBEDO}, capi.PLT_NOT_SUPPORTED),
                     ({"debug_view": capi.DEBUG_VIEW_ROUGHNESS}, capi.PLT_NOT_SUPPORTED)):
        o = _options(**kw)
        h = C.c_void_p()
        assert lib.plt_create(C.byref(o), C.byref(h)) == want, kw
