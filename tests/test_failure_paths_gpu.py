"""The device-side error paths, exercised without faulting the GPU.

Every device wait in the library is bounded and every traversal stack has a fixed depth; when a
bound trips, the kernel records it in the context's status word and returns, and plt_check_status
reports PLT_QUEUE_TIMEOUT.  Two failure-injection option flags make the bounds trip on purpose:
PLT_OPTION_FAULT_COPY_WAIT gives the BSDF shade kernel's wait for its spectral-table copy a zero
poll budget, and PLT_OPTION_FAULT_SHORT_STACK gives plt_trace_* a 2-entry stack.  The tests check
that the status comes back, that the CUDA context stays usable, and that the next normal call on
the same device gives correct results.
"""
import numpy as np
import pytest

import oracle
import parity
from pltfalcor_gb300 import capi
from pltfalcor_gb300 import scene as S
from pltfalcor_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    return torch


def test_copy_wait_timeout_reported(torch_cuda, product_lib, oracle_lib, profiles):
    from pltfalcor_gb300.bsdf import DeviceBatch, PLTContext
    wl = W.mixed_material_batch(n=8 * 1024, profiles=profiles[0])
    ops = capi.OP_EVAL | capi.OP_PDF | capi.OP_SAMPLE
    bad = PLTContext({"flags": capi.OPTION_FAULT_COPY_WAIT})
    bad.set_spectral_profiles(profiles[0])
    bad.set_materials(wl.records)
    b = DeviceBatch(wl)
    b.out_pdf.fill_(-7.0)
    bad.batch(b.queries(), b.results(ops), ops)
    assert bad.check_status() == capi.PLT_QUEUE_TIMEOUT
    # the shade CTAs gave up before shading: no output was written
    assert bool((b.out_pdf == -7.0).all())
    # the status word was cleared by the check
    assert bad.check_status() == capi.PLT_OK
    bad.close()
    # the next normal call on the device is correct
    good = PLTContext()
    good.set_spectral_profiles(profiles[0])
    good.set_materials(wl.records)
    g = DeviceBatch(wl)
    good.batch(g.queries(), g.results(ops), ops)
    assert good.check_status() == capi.PLT_OK
    got = g.fetch()
    o32 = oracle.run(wl, ops=ops, precision=32)
    o64 = oracle.run(wl, ops=ops, precision=64)
    orr = [oracle.run(wl, ops=ops, precision=16, sr_seed=s) for s in (1, 2)]
    errs = parity.compare(got, o32, wl.n, wl.hwss, ops, o64, orr)
    assert not parity.check(errs, max_bad_frac=2e-3), parity.summarize(errs)
    good.close()


def _trace(ctx, torch, o, d):
    dev = torch.device("cuda")
    go = torch.from_numpy(np.ascontiguousarray(o, np.float32)).to(dev)
    gd = torch.from_numpy(np.ascontiguousarray(d, np.float32)).to(dev)
    n = len(o) // 3
    prim = torch.zeros(n, dtype=torch.int32, device=dev)
    ctx.trace_closest(ctx.rays(go, gd), prim)
    st = ctx.check_status()
    return st, prim.cpu().numpy().view(np.uint32)


def test_short_stack_overflow_reported(torch_cuda, product_lib, oracle_lib):
    from pltfalcor_gb300.bsdf import PLTContext
    sc = S.small_scene()
    o, d = S.random_rays(4096, 21, sc.bounds)
    bad = PLTContext({"flags": capi.OPTION_FAULT_SHORT_STACK})
    bad.set_scene(sc.vertices, sc.indices, sc.tri_material)
    st, _ = _trace(bad, torch_cuda, o, d)
    assert st == capi.PLT_QUEUE_TIMEOUT
    bad.close()
    good = PLTContext()
    good.set_scene(sc.vertices, sc.indices, sc.tri_material)
    st, prim = _trace(good, torch_cuda, o, d)
    assert st == capi.PLT_OK
    ref, _, _ = oracle.trace_brute(sc.triangle_vertices(), o, d)
    assert np.array_equal(prim, ref.view(np.uint32))
    good.close()
