"""Chi-square tests of the oracle's samplers against their own densities (tests/chi2.py): the
histogram of 2^17 non-delta samples per case in equal-area bins of the projected disk.  This pins
the oracle's sampling and the test's density rules on the CPU; tests/test_chi2_gpu.py applies the
same test to the library's samplers."""
import pytest

import chi2

P_MIN = 1e-3   # per test (14 cases): a family-wise false-failure rate of about 1 %


@pytest.mark.parametrize("case", chi2.cases(), ids=[c[0] for c in chi2.cases()])
@pytest.mark.parametrize("wi_deg", chi2.WI)
def test_oracle_sampler_chi2(oracle_lib, case, wi_deg):
    import oracle
    name, factory, family, kind, k = case
    prof, _ = oracle.standard_profiles()
    wi = chi2.direction(*wi_deg)
    run = lambda wl, ops: oracle.run(wl, ops=ops)
    p, stat, dof, used = chi2.run_case(run, factory(), prof, family, kind, k, wi, 1 << 17)
    assert used > 4000, (name, used)   # the dielectric keeps about 4 % (its reflectance) as scatter reflections
    assert p > P_MIN, "%s wi %s: chi2 %.1f dof %d p %.3g (%d samples)" % (name, wi_deg, stat, dof, p, used)


def test_chi2_rejects_a_wrong_density(oracle_lib):
    """The test's power: the fractal conductor's samples against pdf() without the 1 / phi_max
    factor of its sampler (the density a sampler that ignored its azimuth limit would have)."""
    import oracle
    name, factory, family, kind, k = chi2.cases()[1]
    prof, _ = oracle.standard_profiles()
    wi = chi2.direction(65.0, 200.0)
    run = lambda wl, ops: oracle.run(wl, ops=ops)
    p, stat, dof, used = chi2.run_case(run, factory(), prof, family, "gauss", k, wi, 1 << 17)
    assert p < 1e-6, (name, p, stat, dof)
