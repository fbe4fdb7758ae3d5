"""The oracle's environment light (oracle/plt_oracle_env.hpp) on the CPU: the lat-long orientation of
EnvMap.eval (world_to_latlong_map; the reference's MathHelpers test checks the same mapping by a
round trip through latlong_map_to_world), the importance map's normalisation, agreement of the
sampler's pdf with evalPdf, the rotation, and the importance-sampled estimate of the map's integral.

Parity of the library's GPU sampler with this oracle is tests/test_envmap_gpu.py.
"""
import numpy as np
import pytest

from pltfalcor_gb300 import scene as S


@pytest.fixture(scope="module")
def orc(oracle_lib):
    import oracle
    return oracle


def latlong_map_to_world(u, v):
    """MathHelpers.slang:120-128."""
    phi = np.pi * (2 * np.clip(u, 0, 1) - 1)
    th = np.pi * np.clip(v, 0, 1)
    return np.stack([np.sin(th) * np.sin(phi), np.cos(th), -np.sin(th) * np.cos(phi)], -1)


def _uniform_dirs(n, seed):
    rng = np.random.default_rng(seed)
    z = rng.uniform(-1, 1, n)
    ph = rng.uniform(0, 2 * np.pi, n)
    s = np.sqrt(1 - z * z)
    return np.stack([s * np.cos(ph), s * np.sin(ph), z], -1).astype(np.float32)


def test_eval_orientation_and_scale(orc):
    """eval at a texel centre's direction returns that texel x intensity x tint."""
    W, H = 64, 32
    img = np.zeros((H, W, 3), np.float32)
    img[..., 0] = np.arange(W)[None, :] + 1
    img[..., 1] = np.arange(H)[:, None] + 1
    img[..., 2] = 1.0
    ys, xs = np.meshgrid(np.arange(2, H - 2), np.arange(W), indexing="ij")
    d = latlong_map_to_world((xs.ravel() + 0.5) / W, (ys.ravel() + 0.5) / H).astype(np.float32)
    env = dict(rgb=img, intensity=2.0, tint=(1.0, 0.5, 0.25))
    out = orc.env_query(env, np.full((len(d), 2), 0.5, np.float32), d)
    want = img[ys.ravel(), xs.ravel()] * np.array([2.0, 1.0, 0.5], np.float32)
    np.testing.assert_allclose(out[:, 8:11], want, rtol=2e-3, atol=2e-3)
    # -z is the map centre, +y the top row
    c = orc.env_query(env, np.zeros((2, 2), np.float32), np.array([[0, 0, -1], [0, 1, 0]], np.float32))
    assert abs(c[0, 8] / 2.0 - (W / 2 + 0.5)) < 0.51 and abs(c[0, 9] - (H / 2 + 0.5)) < 0.51
    assert abs(c[1, 9] - 1.0) < 1e-3


def test_constant_map_is_uniform(orc):
    env = dict(rgb=np.full((16, 32, 3), 0.7, np.float32))
    u = np.random.default_rng(1).uniform(0, 1, (4096, 2)).astype(np.float32)
    out = orc.env_query(env, u, _uniform_dirs(4096, 2))
    np.testing.assert_allclose(out[:, 3], 1 / (4 * np.pi), rtol=1e-5)
    np.testing.assert_allclose(out[:, 7], 1 / (4 * np.pi), rtol=1e-5)
    np.testing.assert_allclose(out[:, 11], 1 / (4 * np.pi), rtol=1e-5)
    np.testing.assert_allclose(np.linalg.norm(out[:, :3], axis=1), 1.0, atol=1e-5)


def test_sample_pdf_matches_eval_pdf_and_integrates(orc):
    env = dict(rgb=S.sky_env(), intensity=1.5)
    n = 1 << 16
    u = np.random.default_rng(3).uniform(0, 1, (n, 2)).astype(np.float32)
    d = _uniform_dirs(n, 4)
    out = orc.env_query(env, u, d)
    np.testing.assert_allclose(np.linalg.norm(out[:, :3], axis=1), 1.0, atol=1e-5)
    # the sample's pdf is evalPdf at its direction (but at texel boundaries of the importance map)
    same = np.isclose(out[:, 3], out[:, 7], rtol=1e-5)
    assert same.mean() > 0.995, same.mean()
    # evalPdf integrates to one over the sphere (uniform directions)
    assert abs(out[:, 11].mean() * 4 * np.pi - 1.0) < 0.02


def test_importance_estimate_of_the_integral(orc):
    """E_q[lum(L) / q] over importance samples equals the map's integral over the sphere, which the
    texel sum gives (lat-long texel solid angles)."""
    img = S.sky_env(width=128, height=64, sun_radiance=20.0)
    W, H = img.shape[1], img.shape[0]
    v0 = np.arange(H) / H
    dOmega = (2 * np.pi / W) * (np.cos(np.pi * v0) - np.cos(np.pi * (v0 + 1.0 / H)))
    lum = img @ np.array([0.2126, 0.7152, 0.0722])
    exact = float((lum * dOmega[:, None]).sum())
    n = 1 << 18
    u = np.random.default_rng(5).uniform(0, 1, (n, 2)).astype(np.float32)
    out = orc.env_query(dict(rgb=img), u)
    est = (out[:, 4:7] @ np.array([0.2126, 0.7152, 0.0722]) / out[:, 3]).mean()
    assert abs(est / exact - 1) < 0.02, (est, exact)


def test_rotation(orc):
    """Rotation (90, 0, 0): toWorld = Rx(90 deg) maps the map's +y to world +z; eval and sample
    directions rotate accordingly."""
    img = S.sky_env(width=64, height=32)
    u = np.random.default_rng(6).uniform(0, 1, (2048, 2)).astype(np.float32)
    d = _uniform_dirs(2048, 7)
    Rx = np.array([[1, 0, 0], [0, 0, -1], [0, 1, 0]], np.float32)
    a = orc.env_query(dict(rgb=img), u, d @ Rx)                  # unrotated, at Rx^T d
    b = orc.env_query(dict(rgb=img, rotation=(90.0, 0.0, 0.0)), u, d)
    np.testing.assert_allclose(b[:, 8:12], a[:, 8:12], rtol=2e-3, atol=1e-4)
    np.testing.assert_allclose(b[:, :3], a[:, :3] @ Rx.T, atol=1e-5)
    np.testing.assert_allclose(b[:, 3], a[:, 3], rtol=1e-5)
