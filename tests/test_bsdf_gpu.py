"""GPU parity of the batched BSDF kernels against the CPU oracle, through the C ABI.

Tolerances are stated in tests/parity.py: 1e-4 relative vs the FP32 oracle, widened per query to
10x the FP32 oracle's own error against the FP64 oracle where the FP32 arithmetic is
ill-conditioned; discrete sample outcomes bit-exact up to a 1e-3 fraction of threshold-straddling
draws.
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

import oracle
import parity
from pltfalcor_gb300 import capi
from pltfalcor_gb300 import materials as M
from pltfalcor_gb300 import workloads as W

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    return torch


@pytest.fixture(scope="module")
def ctx(torch_cuda, product_lib, profiles):
    from pltfalcor_gb300.bsdf import PLTContext
    c = PLTContext()
    c.set_spectral_profiles(profiles[0])
    yield c
    c.close()


def run_gpu(ctx, wl, ops=None, rng_offset=0):
    from pltfalcor_gb300.bsdf import DeviceBatch
    ops = wl.ops if ops is None else ops
    ctx.set_materials(wl.records)
    b = DeviceBatch(wl)
    ctx.batch(b.queries(rng_offset=rng_offset), b.results(ops), ops)
    st = ctx.check_status()
    assert st == capi.PLT_OK, capi.STATUS_NAMES[st]
    return b.fetch()


def oracles(wl, ops=0xF, **kw):
    """FP32 oracle, FP64 oracle and the FP32 oracle with random rounding (conditioning)."""
    return (oracle.run(wl, ops=ops, precision=32, **kw), oracle.run(wl, ops=ops, precision=64),
            [oracle.run(wl, ops=ops, precision=16, sr_seed=s, **kw) for s in (1, 2)])


def assert_parity(gpu, ora, wl, ops, label):
    errs = parity.compare(gpu, ora[0], wl.n, wl.hwss, ops, ora[1], ora[2])
    types = np.asarray(wl.records["type"])[wl.material]
    fails = []
    for t in np.unique(types):
        f = parity.check(errs, sel=types == t)
        fails += ["%s %s: %s" % (label, M.TYPE_NAMES.get(int(t), t), x) for x in f]
    assert not fails, "\n".join(fails)
    return errs


def test_rough_dielectric_parity(ctx, profiles):
    wl = W.rough_dielectric_batch(profiles=profiles[0])
    g = run_gpu(ctx, wl, ops=0xF)
    assert_parity(g, oracles(wl), wl, 0xF, "rough_dielectric_65536")


@pytest.mark.parametrize("hwss,n", [(1, 8 * 16384), (4, 8 * 4096), (2, 8 * 1024), (3, 8 * 1024), (8, 8 * 1024)])
def test_mixed_material_parity(ctx, profiles, hwss, n):
    wl = W.mixed_material_batch(n=n, profiles=profiles[0], hwss=hwss)
    g = run_gpu(ctx, wl, ops=0xF)
    assert_parity(g, oracles(wl), wl, 0xF, "mixed_hwss%d" % hwss)


def test_transmission_and_grazing_cases(ctx, profiles):
    """Lower-hemisphere directions (transmission), grazing angles and all-lobe evaluation."""
    n = 8 * 4096
    wl = W.mixed_material_batch(n=n, profiles=profiles[0])
    rng = W.CounterRNG(77, n)
    v = wl.v.reshape(3, n).copy()
    w = wl.w.reshape(3, n).copy()
    flip = rng.uniform() < 0.5
    w[2, flip] *= -1
    graze = rng.uniform() < 0.2
    v[2, graze] = np.float32(1e-3)
    v[:, graze] /= np.linalg.norm(v[:, graze], axis=0)
    wl.v, wl.w = np.ascontiguousarray(v.reshape(-1)), np.ascontiguousarray(w.reshape(-1))
    wl.lobe = np.where(rng.uniform() < 0.3, np.uint32(0xFFFF), wl.lobe).astype(np.uint32)
    g = run_gpu(ctx, wl, ops=0xF)
    assert_parity(g, oracles(wl), wl, 0xF, "transmission_grazing")


def test_golden_fixtures(ctx, profiles):
    import golden_cases
    for name, wl in golden_cases.cases(profiles[0]).items():
        ref = np.load(os.path.join(GOLDEN, name + ".npz"))
        keys = ("stokes", "coherence", "pdf", "lambda_pdf", "sample_wo", "sample_pdf", "sample_weight", "sample_lobe", "sample_valid")
        o32 = {k: ref[k + "_fp32"] for k in keys}
        o64 = {k: ref[k + "_fp64"] for k in keys}
        orr = [{k: ref[k + "_rr"] for k in keys}, {k: ref[k + "_rr2"] for k in keys}]
        g = run_gpu(ctx, wl, ops=0xF)
        errs = parity.compare(g, o32, wl.n, wl.hwss, 0xF, o64, orr)
        fails = parity.check(errs, max_bad_frac=2e-3)
        assert not fails, (name, fails)


def grazing_conductor_batch(profiles, n=3 * 8192, seed=7):
    """Conductor, coated-conductor and grated-conductor queries of the mixed-material batch with
    both directions at grazing incidence (cos theta uniform in [0.001, 0.1], random azimuths)."""
    wl = W.mixed_material_batch(n=8 * n, profiles=profiles)
    types = np.asarray(wl.records["type"])[wl.material]
    idx = np.nonzero(np.isin(types, [M.CONDUCTOR, M.COATED_CONDUCTOR, M.GRATED_CONDUCTOR]))[0][:n]
    g = wl.subset(idx)
    rng = np.random.default_rng(seed)
    for key, sgn in (("v", 1.0), ("w", 1.0)):
        c = rng.uniform(0.001, 0.1, g.n)
        phi = rng.uniform(0.0, 2 * np.pi, g.n)
        s = np.sqrt(1 - c * c)
        setattr(g, key, np.ascontiguousarray(np.stack([s * np.cos(phi), s * np.sin(phi), sgn * c]).astype(np.float32).reshape(-1)))
    return g


def test_fp64_error_report(ctx, profiles, tmp_path):
    """Error of the GPU (FP32) and of the FP32 oracle against the FP64 oracle, per material, and the
    share of queries whose GPU result differs from the FP32 oracle's by more than a raw 1e-4;
    then, at grazing incidence on the conductor materials, the same errors with and without
    PLT_OPTION_FP64_CONDUCTOR_GRAZING.  PLT_FP64_REPORT=path writes the report as JSON."""
    from pltfalcor_gb300.bsdf import PLTContext
    wl = W.mixed_material_batch(n=8 * 8192, profiles=profiles[0])
    g = run_gpu(ctx, wl, ops=0xF)
    o32 = oracle.run(wl, ops=0xF, precision=32)
    o64 = oracle.run(wl, ops=0xF, precision=64)
    types = np.asarray(wl.records["type"])[wl.material]
    report = {"workload": "mixed_material_batch 65536 queries (seed 1), eval + pdf + sample + lambdaPdf, HWSS 1",
              "tolerance": "raw relative error 1e-4 (errors as tests/parity.py defines them)", "materials": {}}
    eg = parity.errors(g, o64, wl.n, 1, 0xF)
    eo = parity.errors(o32, o64, wl.n, 1, 0xF)
    e32 = parity.errors(g, o32, wl.n, 1, 0xF)
    for t in np.unique(types):
        sel = types == t
        name = M.TYPE_NAMES[int(t)]
        gs, os_ = parity.summarize(eg, sel=sel), parity.summarize(eo, sel=sel)
        raw = {k: float((v[sel] > parity.TOL).mean()) for k, v in e32.items() if v.dtype != bool}
        report["materials"][name] = {
            "queries": int(sel.sum()),
            "gpu_fp32_vs_fp64": {k: {q: v[q] for q in ("p50", "p99", "max")} for k, v in gs.items() if "p99" in v},
            "oracle_fp32_vs_fp64": {k: {q: v[q] for q in ("p50", "p99", "max")} for k, v in os_.items() if "p99" in v},
            "gpu_vs_oracle_fp32_frac_above_1e-4": raw}
        for k in ("stokes", "pdf"):
            # the GPU is no further from FP64 than the FP32 reference arithmetic, within 10x at p99
            gp, op = gs[k]["p99"], os_[k]["p99"]
            assert gp <= max(10 * op, 1e-5), (name, k, gp, op)
    # grazing incidence on conductors: the FP64 Fresnel option against the FP32 default
    gw = grazing_conductor_batch(profiles[0])
    gtypes = np.asarray(gw.records["type"])[gw.material]
    g64 = oracle.run(gw, ops=1, precision=64)
    plain = run_gpu(ctx, gw, ops=1)
    c2 = PLTContext({"flags": capi.OPTION_FP64_CONDUCTOR_GRAZING})
    c2.set_spectral_profiles(profiles[0])
    opt = run_gpu(c2, gw, ops=1)
    c2.close()
    ep, eopt = parity.errors(plain, g64, gw.n, 1, 1), parity.errors(opt, g64, gw.n, 1, 1)
    graz = {}
    for t in np.unique(gtypes):
        sel = gtypes == t
        graz[M.TYPE_NAMES[int(t)]] = {
            "queries": int(sel.sum()),
            "gpu_fp32_vs_fp64_stokes": {q: float(np.quantile(ep["stokes"][sel], x)) for q, x in (("p50", .5), ("p99", .99))} |
                                       {"max": float(ep["stokes"][sel].max())},
            "gpu_fp64_grazing_option_vs_fp64_stokes": {q: float(np.quantile(eopt["stokes"][sel], x)) for q, x in (("p50", .5), ("p99", .99))} |
                                                      {"max": float(eopt["stokes"][sel].max())}}
    report["grazing_conductors"] = {"workload": "conductor, coated conductor and grated conductor queries, both directions with "
                                                "cos theta in [0.001, 0.1], eval, HWSS 1; option PLT_OPTION_FP64_CONDUCTOR_GRAZING "
                                                "(FP64 complex Fresnel below cos theta 0.1)", "materials": graz}
    out = os.environ.get("PLT_FP64_REPORT")
    if out:
        with open(out, "w") as f:
            json.dump(report, f, indent=1)


def test_fp64_conductor_grazing_option(torch_cuda, product_lib, profiles):
    """PLT_OPTION_FP64_CONDUCTOR_GRAZING against the FP32 oracle with the same option, at grazing
    incidence on every conductor material and on the whole mixed batch (where it is inactive for
    most queries)."""
    from pltfalcor_gb300.bsdf import PLTContext
    c = PLTContext({"flags": capi.OPTION_FP64_CONDUCTOR_GRAZING})
    c.set_spectral_profiles(profiles[0])
    for wl in (grazing_conductor_batch(profiles[0], n=3 * 2048), W.mixed_material_batch(n=8 * 2048, profiles=profiles[0])):
        g = run_gpu(c, wl, ops=0xF)
        o = oracle.run(wl, ops=0xF, precision=32, fp64_conductor_grazing=True)
        o64 = oracle.run(wl, ops=0xF, precision=64)
        orr = [oracle.run(wl, ops=0xF, precision=16, sr_seed=s, fp64_conductor_grazing=True) for s in (1, 2)]
        errs = parity.compare(g, o, wl.n, 1, 0xF, o64, orr)
        assert not parity.check(errs), parity.summarize(errs)
    c.close()


def test_fp64_multilayer_option(torch_cuda, product_lib, profiles):
    from pltfalcor_gb300.bsdf import PLTContext
    c = PLTContext(fp64_multilayer=True)
    c.set_spectral_profiles(profiles[0])
    wl = W.mixed_material_batch(n=8 * 2048, profiles=profiles[0])
    g = run_gpu(c, wl, ops=1)
    o = oracle.run(wl, ops=1, precision=32, fp64_multilayer=True)
    o64 = oracle.run(wl, ops=1, precision=64)
    orr = [oracle.run(wl, ops=1, precision=16, sr_seed=s, fp64_multilayer=True) for s in (1, 2)]
    ml = np.asarray(wl.records["type"])[wl.material] == M.MULTILAYERED_STACK
    errs = parity.compare(g, o, wl.n, 1, 1, o64, orr)
    assert not parity.check(errs, sel=ml)
    c.close()


def test_full_size_properties(ctx, profiles, torch_cuda):
    """The 2^22 mixed-material batch: finite outputs, polarisation bound, exact zeros above
    720 nm, run-to-run determinism and chunked == single launch."""
    torch = torch_cuda
    from pltfalcor_gb300.bsdf import DeviceBatch
    wl = W.mixed_material_batch(n=1 << 22, profiles=profiles[0])
    ctx.set_materials(wl.records)
    b = DeviceBatch(wl)
    ctx.batch(b.queries(), b.results(0xF), 0xF)
    assert ctx.check_status() == capi.PLT_OK
    r1 = b.fetch()
    ctx.batch(b.queries(), b.results(0xF), 0xF)
    r2 = b.fetch()
    for k in r1:
        assert np.array_equal(r1[k].view(np.uint32), r2[k].view(np.uint32)), k
    S = r1["stokes"].reshape(4, -1).astype(np.float64)
    assert np.isfinite(S).all() and np.isfinite(r1["pdf"]).all() and np.isfinite(r1["sample_pdf"]).all()
    types = np.asarray(M.BENCH_TYPES)[wl.meta["types"]]
    fres = np.isin(types, [M.DIELECTRIC, M.CONDUCTOR, M.MULTILAYERED_STACK, M.GRATED_CONDUCTOR, M.GRATED_OPAQUE_DIELECTRIC])
    dop = np.sqrt(S[1] ** 2 + S[2] ** 2 + S[3] ** 2)
    assert (dop[fres] <= S[0, fres] * (1 + 1e-4) + 1e-30).all()
    # rgbToSpectrum is zero for lambda >= 720 nm: every m00-weighted material returns exact zeros
    hi = wl.wavelengths >= 720.0
    m00w = np.isin(types, [M.DIELECTRIC, M.CONDUCTOR, M.GRATED_CONDUCTOR, M.GRATED_OPAQUE_DIELECTRIC])
    assert (S[:, hi & m00w] == 0).all()
    # the second half as its own batch with rng_offset == the same results (streams are per query index)
    half = wl.n // 2
    sub = wl.subset(np.arange(half, wl.n))
    bs = DeviceBatch(sub)
    ctx.batch(bs.queries(rng_offset=half), bs.results(0xF), 0xF)
    rs = bs.fetch()
    assert np.array_equal(rs["sample_lobe"], r1["sample_lobe"][half:])
    assert np.array_equal(rs["sample_pdf"].view(np.uint32), r1["sample_pdf"][half:].view(np.uint32))
    assert np.array_equal(rs["stokes"].reshape(4, -1).view(np.uint32), r1["stokes"].reshape(4, -1)[:, half:].view(np.uint32))


def test_status_on_bad_inputs(ctx, profiles, torch_cuda):
    torch = torch_cuda
    from pltfalcor_gb300.bsdf import DeviceBatch
    wl = W.mixed_material_batch(n=8 * 256, profiles=profiles[0])
    ctx.set_materials(wl.records)
    bad = wl.material.copy()
    bad[5] = len(wl.records) + 10
    wl2 = W.Workload("bad", wl.n, 1, bad, wl.v, wl.w, wl.lobe, wl.wavelengths, wl.stokes, wl.coherence, wl.records, wl.profiles, 0xF)
    b = DeviceBatch(wl2)
    ctx.batch(b.queries(), b.results(0xF), 0xF)
    assert ctx.check_status() == capi.PLT_BAD_MATERIAL
    r = b.fetch()
    assert (r["stokes"].reshape(4, -1)[:, 5] == 0).all() and r["sample_valid"][5] == 0
    # a NaN direction is reported
    v = wl.v.copy()
    v[7] = np.nan
    wl3 = W.Workload("nan", wl.n, 1, wl.material, v, wl.w, wl.lobe, wl.wavelengths, wl.stokes, wl.coherence, wl.records, wl.profiles, 0xF)
    b3 = DeviceBatch(wl3)
    ctx.batch(b3.queries(), b3.results(0x1), 0x1)
    assert ctx.check_status() == capi.PLT_NAN_INPUT
    # invalid arguments are rejected on the host, before any launch
    q = b.queries()
    q.hwss = 0
    with pytest.raises(capi.PLTError) as e:
        ctx.batch(q, b.results(1), 1)
    assert e.value.status == capi.PLT_INVALID_ARG
    q = b.queries()
    q.v = C.c_void_p(q.v + 4)  # misaligned plane
    with pytest.raises(capi.PLTError):
        ctx.batch(q, b.results(1), 1)
    with pytest.raises(capi.PLTError):
        ctx.batch(b.queries(), b.results(1), 0x10)
    # unknown material types and out-of-range spectral ids are rejected by plt_set_materials
    recs = wl.records.copy()
    recs["type"][0] = 99
    with pytest.raises(capi.PLTError):
        ctx.set_materials(recs)
    recs = wl.records.copy()
    cond = np.where(recs["type"] == M.CONDUCTOR)[0][0]
    recs["ior_n_spectral_id"][cond] = 50
    with pytest.raises(capi.PLTError):
        ctx.set_materials(recs)
