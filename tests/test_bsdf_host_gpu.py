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


@pytest.mark.parametrize("n,hwss,ops,pin", [((1 << 20) + (1 << 18) + 7, 1, capi.OP_EVAL | capi.OP_SAMPLE | capi.OP_PDF, True),
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
    for rep in range(2):
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
