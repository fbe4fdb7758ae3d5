"""plt_bsdf_batch_host (host queries and results, chunked copy/compute pipeline) against
plt_bsdf_batch on device-resident buffers: the results must be bit-identical, including a final
partial chunk of a size that is not a multiple of 4, pageable (unpinned) host memory, a subset of
ops and HWSS 4, and repeated calls that reuse the staging slots."""
import numpy as np
import pytest

from pltfalcor_gb300 import capi, spectra
from pltfalcor_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    return torch


# the first case spans two 2^21-query chunks (the second partial, not a multiple of 4, shaded by
# the small-batch schedule when short); three calls walk the four staging slots round
@pytest.mark.parametrize("n,hwss,ops,pin", [((1 << 21) + (1 << 18) + 7, 1, capi.OP_EVAL | capi.OP_SAMPLE | capi.OP_PDF, True),
                                            ((1 << 21) + 4100, 1, capi.OP_EVAL | capi.OP_PDF, True),
                                            (300_001, 4, capi.OP_ALL, False), (4096, 2, capi.OP_SAMPLE, True)])
def test_host_batch_equals_device_batch(torch_cuda, product_lib, n, hwss, ops, pin):
    from pltfalcor_gb300.bsdf import DeviceBatch, PLTContext
    prof, _ = spectra.standard_profiles()
    wl = W.mixed_material_batch(n=(n + 7) // 8 * 8, profiles=prof, hwss=hwss)
    if wl.n != n:
        wl = wl.subset(np.arange(n))
    ctx = PLTContext()
    ctx.set_spectral_profiles(prof)
    ctx.set_materials(wl.records)
    d = DeviceBatch(wl)
    ctx.batch(d.queries(rng_offset=11), d.results(ops), ops)
    torch_cuda.cuda.synchronize()
    ref = d.fetch()
    h = DeviceBatch(wl, device="cpu", pin=pin)
    for rep in range(3):
        ctx.batch_host(h.queries(rng_offset=11), h.results(ops), ops)
        torch_cuda.cuda.synchronize()
    assert ctx.check_status() == capi.PLT_OK
    got = h.fetch()
    keys = []
    if ops & capi.OP_EVAL:
        keys += ["stokes", "coherence"]
    if ops & capi.OP_PDF:
        keys += ["pdf"]
    if ops & capi.OP_LAMBDA_PDF:
        keys += ["lambda_pdf"]
    if ops & capi.OP_SAMPLE:
        keys += ["sample_wo", "sample_pdf", "sample_weight", "sample_lobe", "sample_valid"]
    for k in keys:
        assert np.array_equal(got[k].view(np.uint32), ref[k].view(np.uint32)), k
    ctx.close()


def test_host_batch_ordered_on_callers_stream(torch_cuda, product_lib):
    """The ordering contract of plt_bsdf_batch_host on one explicit stream, with no device-wide
    synchronisation: a device batch and then the async device-to-host copies that produce the host
    inputs are queued on `s` just before the call (behind a spin of a few milliseconds), so a
    pipeline that started reading before the work queued on `s` finished would read zeros.  Only `s`
    is synchronised, once, after a device batch queued behind the call; the host results must equal
    the first device batch bit for bit, and the last device batch must equal it too (no shared
    scratch between the pipeline and plt_bsdf_batch)."""
    torch = torch_cuda
    from pltfalcor_gb300.bsdf import DeviceBatch, PLTContext
    prof, _ = spectra.standard_profiles()
    n = (1 << 21) + 4100   # two chunks, the second short
    wl = W.mixed_material_batch(n=(n + 7) // 8 * 8, profiles=prof)
    wl = wl.subset(np.arange(n))
    ops = capi.OP_EVAL | capi.OP_SAMPLE | capi.OP_PDF
    ctx = PLTContext()
    ctx.set_spectral_profiles(prof)
    ctx.set_materials(wl.records)
    d = DeviceBatch(wl)
    d2 = DeviceBatch(wl)
    h = DeviceBatch(wl, device="cpu", pin=True)
    pairs = [(d.material, h.material), (d.v, h.v), (d.w, h.w), (d.lobe, h.lobe), (d.wavelengths, h.wavelengths),
             (d.stokes, h.stokes), (d.coherence, h.coherence)]
    for _, ht in pairs:
        ht.zero_()
    torch.cuda.synchronize()   # set-up uploads only; nothing below synchronises the device
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ctx.batch(d.queries(rng_offset=5), d.results(ops), ops, s)
        torch.cuda._sleep(20_000_000)
        for dt, ht in pairs:
            ht.copy_(dt, non_blocking=True)
        ctx.batch_host(h.queries(rng_offset=5), h.results(ops), ops, s)
        ctx.batch(d2.queries(rng_offset=5), d2.results(ops), ops, s)
    assert ctx.check_status(s) == capi.PLT_OK   # synchronises `s` only
    ref, got, again = d.fetch(), h.fetch(), d2.fetch()
    for k in ["stokes", "coherence", "pdf", "sample_wo", "sample_pdf", "sample_weight", "sample_lobe", "sample_valid"]:
        assert np.array_equal(got[k].view(np.uint32), ref[k].view(np.uint32)), k
        assert np.array_equal(again[k].view(np.uint32), ref[k].view(np.uint32)), k
    ctx.close()


def test_host_batch_slots_grow_between_calls(torch_cuda, product_lib):
    """One context, calls of growing then shrinking size: the staging slots are sized for the
    first call's chunk and reallocated (after the pipeline drains) when a later call's chunk is
    larger; every call's results equal plt_bsdf_batch's bit for bit."""
    from pltfalcor_gb300.bsdf import DeviceBatch, PLTContext
    prof, _ = spectra.standard_profiles()
    ops = capi.OP_EVAL | capi.OP_SAMPLE | capi.OP_PDF
    ctx = PLTContext()
    ctx.set_spectral_profiles(prof)
    full = W.mixed_material_batch(n=(1 << 21) + 104, profiles=prof)
    ctx.set_materials(full.records)
    for n, off in ((4096, 3), ((1 << 21) + 100, 5), (70_001, 7)):
        wl = full.subset(np.arange(n))
        d = DeviceBatch(wl)
        ctx.batch(d.queries(rng_offset=off), d.results(ops), ops)
        torch_cuda.cuda.synchronize()
        ref = d.fetch()
        h = DeviceBatch(wl, device="cpu", pin=True)
        ctx.batch_host(h.queries(rng_offset=off), h.results(ops), ops)
        torch_cuda.cuda.synchronize()
        assert ctx.check_status() == capi.PLT_OK
        got = h.fetch()
        for k in ["stokes", "coherence", "pdf", "sample_wo", "sample_pdf", "sample_weight", "sample_lobe", "sample_valid"]:
            assert np.array_equal(got[k].view(np.uint32), ref[k].view(np.uint32)), (n, k)
    ctx.close()
