"""Chi-square tests of the library's samplers (plt_bsdf_batch sample) against their own densities
(tests/chi2.py), 2^20 samples per case, through the C ABI on the GPU: the densities come from the
library's pdf on the bin grid, so a sampling mistake that the oracle shares would still show."""
import pytest

import chi2
from pltfalcor_gb300 import capi

pytestmark = pytest.mark.gpu

P_MIN = 1e-3


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    return torch


@pytest.fixture(scope="module")
def gpu_run(torch_cuda, product_lib, profiles):
    from pltfalcor_gb300.bsdf import DeviceBatch, PLTContext
    ctx = PLTContext()
    ctx.set_spectral_profiles(profiles[0])

    def run(wl, ops):
        ctx.set_materials(wl.records)
        b = DeviceBatch(wl)
        ctx.batch(b.queries(), b.results(ops), ops)
        assert ctx.check_status() == capi.PLT_OK
        return b.fetch()
    yield run
    ctx.close()


@pytest.mark.parametrize("case", chi2.cases(), ids=[c[0] for c in chi2.cases()])
@pytest.mark.parametrize("wi_deg", chi2.WI)
def test_library_sampler_chi2(gpu_run, profiles, case, wi_deg):
    name, factory, family, kind, k = case
    wi = chi2.direction(*wi_deg)
    p, stat, dof, used = chi2.run_case(gpu_run, factory(), profiles[0], family, kind, k, wi, 1 << 20, frame=3)
    assert used > 30000, (name, used)
    assert p > P_MIN, "%s wi %s: chi2 %.1f dof %d p %.3g (%d samples)" % (name, wi_deg, stat, dof, p, used)
