"""Known-answer tests pinning the CPU oracle (runs without a GPU).

The reference ships no PLT golden vectors, so the oracle is pinned by closed forms: Fresnel at
normal incidence and Snell's law, the textbook complex conductor Fresnel, the grating equation,
the published SplitMix64 sequence, an independent xoshiro128** implementation, binary16 decoding,
the rgbToSpectrum basis, the multilayer stack with zero layers, degree of polarisation after
Fresnel-only interactions, and the committed fixtures of its own outputs.
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle
from pltfalcor_gb300 import materials as M
from pltfalcor_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_fresnel_normal_incidence(oracle_lib):
    out = (C.c_float * 5)()
    for n in (1.2, 1.5, 2.4):
        oracle_lib.plto_fresnel_dielectric(1.0, n, out)
        rs, rp = out[0], out[1]
        assert abs(rs - (1 - n) / (1 + n)) < 1e-6
        assert abs(rp - (n - 1) / (n + 1)) < 1e-6
        assert abs(0.5 * (rs * rs + rp * rp) - ((n - 1) / (n + 1)) ** 2) < 1e-6


def test_fresnel_snell_and_energy(oracle_lib):
    out = (C.c_float * 5)()
    for cos_i in (0.9, 0.6, 0.2):
        for n in (1.33, 1.5):
            oracle_lib.plto_fresnel_dielectric(cos_i, n, out)
            rs, rp, ts, tp, ct = out[:]
            sin_t = np.sqrt(1 - cos_i ** 2) / n
            assert abs(-ct - np.sqrt(1 - sin_t ** 2)) < 1e-6  # transmitted cosine, opposite side
            # energy conservation per polarisation: r^2 + t^2 = 1 (t includes the impedance factor)
            assert abs(rs * rs + ts * ts - 1) < 1e-5
            assert abs(rp * rp + tp * tp - 1) < 1e-5


def test_conductor_fresnel_textbook(oracle_lib):
    out = (C.c_double * 4)()
    for n, k in ((0.18, 3.4), (1.2, 7.0), (0.27, 2.8)):
        eta = complex(n, k)
        for cos_i in (1.0, 0.7, 0.3, 0.05):
            oracle_lib.plto_fresnel_conductor(cos_i, n, k, out)
            s2 = 1 - cos_i ** 2
            root = np.sqrt(eta * eta - s2)
            rs = (cos_i - root) / (cos_i + root)
            rp = (eta * eta * cos_i - root) / (eta * eta * cos_i + root)
            assert abs(complex(out[0], out[1]) - rs) < 1e-12
            assert abs(complex(out[2], out[3]) - rp) < 1e-12


def test_grating_equation(oracle_lib):
    out = (C.c_float * 3)()
    for th_i in (0.0, 0.3, 0.8):
        wi = (np.sin(th_i), 0.0, np.cos(th_i))
        for m in (-2, -1, 1, 2):
            lam, pitch = 0.55, 2.0
            oracle_lib.plto_diffract(wi[0], wi[1], wi[2], m, 0, lam, 1 / pitch, 0.0, out)
            s_o = m * lam / pitch - np.sin(th_i)
            if abs(s_o) <= 1:
                assert abs(out[0] - s_o) < 1e-6 and abs(out[1]) < 1e-7
                assert abs(np.linalg.norm(out[:]) - 1) < 1e-6
            else:
                assert out[:] == [0.0, 0.0, 0.0]


def test_splitmix64_published_vector():
    # SplitMix64 reference outputs for seed 1234567 (Vigna, splitmix64.c)
    st = np.array([1234567], dtype=np.uint64)
    outs = []
    with np.errstate(over="ignore"):
        for _ in range(3):
            st, z = W._splitmix64(st)
            outs.append(int(z[0]))
    assert outs == [6457827717110365317, 3203168211198807973, 9817491932198370423]


def _xoshiro128ss_py(px, py, frame, count):
    """Independent pure-Python restatement of the published SplitMix64 + xoshiro128** algorithms."""
    M64 = (1 << 64) - 1

    def il(v):
        v &= 0xFFFF
        out = 0
        for b in range(16):
            out |= ((v >> b) & 1) << (2 * b)
        return out
    s = ((frame << 32) | (il(px) | (il(py) << 1))) & M64

    def sm():
        nonlocal s
        s = (s + 0x9E3779B97F4A7C15) & M64
        z = s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M64
        return z ^ (z >> 31)
    a, b = sm(), sm()
    st = [a & 0xFFFFFFFF, a >> 32, b & 0xFFFFFFFF, b >> 32]
    rot = lambda x, k: ((x << k) | (x >> (32 - k))) & 0xFFFFFFFF
    res = []
    for _ in range(count):
        r = (rot((st[0] * 5) & 0xFFFFFFFF, 7) * 9) & 0xFFFFFFFF
        t = (st[1] << 9) & 0xFFFFFFFF
        st[2] ^= st[0]; st[3] ^= st[1]; st[1] ^= st[2]; st[0] ^= st[3]
        st[2] ^= t
        st[3] = rot(st[3], 11)
        res.append(r)
    return res


@pytest.mark.parametrize("px,py,frame", [(0, 0, 0), (3, 5, 9), (65535, 1, 7), (1000, 64, 123456)])
def test_rng_streams_match(oracle_lib, px, py, frame):
    ref = _xoshiro128ss_py(px, py, frame, 16)
    assert list(oracle.rng_stream(px, py, frame, 16)) == ref
    # the workload generator (numpy) draws the same stream for query index px + 65536 py
    r = W.CounterRNG(frame, 1, offset=px + 65536 * py)
    assert [int(r.next_u32()[0]) for _ in range(16)] == ref


def _tea_py(v0, v1, key, rounds):
    """Independent restatement of the published TEA encryption (Wheeler & Needham 1994)."""
    M = 0xFFFFFFFF
    s = 0
    for _ in range(rounds):
        s = (s + 0x9E3779B9) & M
        v0 = (v0 + ((((v1 << 4) & M) + key[0]) ^ (v1 + s) ^ ((v1 >> 5) + key[1]))) & M
        v1 = (v1 + ((((v0 << 4) & M) + key[2]) ^ (v0 + s) ^ ((v0 >> 5) + key[3]))) & M
    return v0, v1


def test_tea_published_vector():
    # the standard TEA test vector: key 0, plaintext 0, 32 cycles
    assert _tea_py(0, 0, [0, 0, 0, 0], 32) == (0x41EA3A0A, 0x94BAA940)


def test_lcg_published_sequence():
    # Numerical Recipes "quick and dirty" generator (a = 1664525, c = 1013904223) from state 0
    s, out = 0, []
    for _ in range(6):
        s = (1664525 * s + 1013904223) & 0xFFFFFFFF
        out.append(s)
    assert out == [0x3C6EF35F, 0x47502932, 0xD1CCF6E9, 0xAAF95334, 0x6252E503, 0x9F2EC686]


@pytest.mark.parametrize("px,py,frame", [(0, 0, 0), (3, 5, 9), (65535, 1, 7), (1000, 64, 123456)])
def test_tiny_rng_stream_matches(oracle_lib, px, py, frame):
    """TinyUniformSampleGenerator: LCG seeded with blockCipherTEA(interleave(pixel), frame).x, 16
    rounds with the key of Utils/Math/HashUtils.slang:59-71."""
    def il(v):
        v &= 0xFFFF
        return sum(((v >> b) & 1) << (2 * b) for b in range(16))
    seed, _ = _tea_py(il(px) | (il(py) << 1), frame, [0xA341316C, 0xC8013EA4, 0xAD90777D, 0x7E95761E], 16)
    ref, s = [], seed
    for _ in range(16):
        s = (1664525 * s + 1013904223) & 0xFFFFFFFF
        ref.append(s)
    assert list(oracle.rng_stream(px, py, frame, 16, tiny=True)) == ref


def test_half_decode(oracle_lib):
    vals = {0x3C00: 1.0, 0x3E00: 1.5, 0x0001: 2.0 ** -24, 0x7BFF: 65504.0, 0xC000: -2.0, 0x0000: 0.0}
    for h, f in vals.items():
        assert oracle_lib.plto_half_to_float(h) == f
    x = np.float32([0.0042, 0.3, 1.38, 2.3, 0.15])
    for v, b in zip(x, M.f16bits(x)):
        assert oracle_lib.plto_half_to_float(int(b)) == float(np.float16(v))


def test_rgb_to_spectrum_white(oracle_lib):
    for wl in (380.0, 450.0, 619.0, 700.0):
        assert abs(oracle_lib.plto_rgb_to_spectrum(1, 1, 1, wl) - 1.0) < 1e-3
    assert oracle_lib.plto_rgb_to_spectrum(1, 1, 1, 725.0) == 0.0
    assert oracle_lib.plto_rgb_to_spectrum(1, 1, 1, 780.0) == 0.0


def test_multilayer_zero_layers_returns_m00(oracle_lib):
    n = 64
    wl = W.rough_dielectric_batch(n=n)
    wl.records = M.multilayered_stack(n, 0, 1.38, 2.3, 0.1, 0.2, albedo=(0.3, 0.6, 0.9))
    wl.lobe = np.full(n, M.LOBE_DELTA_R, np.uint32)
    res = oracle.run(wl, ops=1)
    S = res["stokes"].reshape(4, n)
    wls = wl.wavelengths
    f16 = lambda v: float(np.float16(v))  # the albedo is stored as binary16
    m00 = np.array([oracle_lib.plto_rgb_to_spectrum(f16(0.3), f16(0.6), f16(0.9), float(x)) for x in wls])
    assert np.allclose(S[0], m00, rtol=1e-6, atol=0)


def test_degree_of_polarisation_fresnel_only(profiles):
    prof, _ = profiles
    wl = W.mixed_material_batch(n=8 * 2048, profiles=prof)
    res = oracle.run(wl, ops=1, precision=64)
    S = res["stokes"].reshape(4, -1).astype(np.float64)
    ty = np.asarray(M.BENCH_TYPES)[wl.meta["types"]]
    dop_ok = np.sqrt(S[1] ** 2 + S[2] ** 2 + S[3] ** 2) <= S[0] * (1 + 1e-6) + 1e-30
    for t in (M.DIELECTRIC, M.CONDUCTOR, M.MULTILAYERED_STACK, M.GRATED_CONDUCTOR, M.GRATED_OPAQUE_DIELECTRIC):
        sel = ty == t
        assert dop_ok[sel].all(), (M.TYPE_NAMES[t], (~dop_ok[sel]).sum())


def test_oracle_matches_golden_fixture(profiles):
    prof, _ = profiles
    import golden_cases
    for name, wl in golden_cases.cases(prof).items():
        ref = np.load(os.path.join(GOLDEN, name + ".npz"))
        for tag, prec, seed in (("fp32", 32, 1), ("fp64", 64, 1), ("rr", 16, 1), ("rr2", 16, 2)):
            res = oracle.run(wl, ops=0xF, precision=prec, sr_seed=seed)
            for k, v in res.items():
                r = ref["%s_%s" % (k, tag)]
                if v.dtype == np.uint32:
                    assert (v == r).all(), (name, prec, k)
                else:
                    assert np.allclose(v, r, rtol=1e-5, atol=1e-30, equal_nan=True), (name, prec, k)


def test_op_counting_build(profiles):
    prof, _ = profiles
    wl = W.mixed_material_batch(n=8 * 256, profiles=prof)
    c = oracle.count_ops(wl, ops=0x7)
    assert set(c) == set(M.BENCH_TYPES)
    for t, v in c.items():
        assert 50 < v["fp"] < 5000 and 5 < v["sfu"] < 500


def test_proposal_oracle_backprop_matches_finite_differences(oracle_lib):
    """The CPU network oracle's back-propagation (double precision, no BF16 rounding) against
    central differences of its own loss, on random parameters and a small batch."""
    import oracle as O
    rng = np.random.default_rng(0)
    p = (rng.standard_normal(11488) * 0.2).astype(np.float32)
    n = 16
    xf = rng.standard_normal((n, 16))
    xf[:, 14:] = 0
    t = rng.uniform(-0.7, 0.7, (n, 2)).astype(np.float32)
    w = rng.uniform(0.5, 1.5, n).astype(np.float32)
    _, g = O.mlp_gradient(p, t, w, x_f64=xf, round_bf16=False)
    for idx in list(rng.integers(0, 11488, 30)) + [11456 + 3, 11456 + 1, 9216 + 5]:
        eps = 1e-3 * max(1.0, abs(float(p[idx])))
        pp, pm = p.copy(), p.copy()
        pp[idx] = np.float32(p[idx] + eps)
        pm[idx] = np.float32(p[idx] - eps)
        lp, _ = O.mlp_gradient(pp, t, w, x_f64=xf, round_bf16=False)
        lm, _ = O.mlp_gradient(pm, t, w, x_f64=xf, round_bf16=False)
        fd = (lp - lm) / (float(pp[idx]) - float(pm[idx]))
        assert abs(fd - g[idx]) <= 1e-3 * max(abs(fd), abs(g[idx]), 1e-4), (idx, fd, g[idx])
