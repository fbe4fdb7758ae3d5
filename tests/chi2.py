"""Chi-square goodness-of-fit of a BSDF sampler against its own density, in the pattern of the
reference's BSDF sampling tests (Source/Tools/FalcorTest/Tests/Scene/Material/BSDFTests.cpp:89-300:
histogram the sampled directions, integrate the density over the same bins, Pearson chi-square with
low-expectation bins pooled).  Used by tests/test_chi2_cpu.py (the oracle's samplers) and
tests/test_chi2_gpu.py (the library's).

Bins: equal-area cells of the projected unit disk (wo.x, wo.y): R2_BINS rings in r^2 x PHI_BINS
sectors.  The test is on the shape of the distribution of the non-delta samples of one lobe family,
conditioned on that family, so the expected counts only need a density up to a constant factor:

  - Gaussian surface (PLTDielectric, GaussianSurface.slang:76-95): wo.xy is drawn from the
    truncated Gaussian that pdf() evaluates, then kept as a reflection with probability
    F(wi, h); pdf(toLight = wi, V = wo) for a reflected wo is (1 - alpha) F(wi, h) g(wo.xy), so the
    density of scatter-reflection samples in the disk is proportional to pdf();
  - fractal surface (FractalSurface.slang:97-129, conductor / opaque dielectric / grated bases):
    zeta = k (wi + wo).xy is drawn with radial CDF 1 - (1 + T f^2)^((1 - gamma) / 2) truncated by M
    and azimuth uniform within +-phi_max(f) around wi's azimuth, so the density in the disk is
    k^2 pi pGF(zeta) / (phi_max(|zeta|) M); pdf() is pGF(zeta) (times a factor constant in wo), so
    the density is proportional to pdf() / phi_max(|zeta|);
  - cosine-weighted hemisphere (PLTDiffuse): uniform in the disk.
"""
import numpy as np

R2_BINS, PHI_BINS, SUB = 16, 32, 12


def direction(theta_deg, phi_deg):
    t, p = np.radians(theta_deg), np.radians(phi_deg)
    return np.array([np.sin(t) * np.cos(p), np.sin(t) * np.sin(p), np.cos(t)])


def histogram(wo_xy):
    r2 = np.clip((wo_xy ** 2).sum(axis=0), 0.0, 1.0 - 1e-12)
    phi = np.mod(np.arctan2(wo_xy[1], wo_xy[0]), 2 * np.pi)
    i = np.minimum((r2 * R2_BINS).astype(np.int64), R2_BINS - 1)
    j = np.minimum((phi / (2 * np.pi) * PHI_BINS).astype(np.int64), PHI_BINS - 1)
    return np.bincount(i * PHI_BINS + j, minlength=R2_BINS * PHI_BINS).astype(np.float64)


def grid_points():
    """SUB x SUB midpoints of every bin in (r^2, phi) (equal weights: the cells are equal-area);
    returns xy [2][bins * SUB^2] with the bin of each point."""
    a = (np.arange(SUB) + 0.5) / SUB
    i, j, u, v = np.meshgrid(np.arange(R2_BINS), np.arange(PHI_BINS), a, a, indexing="ij")
    r2 = (i + u) / R2_BINS
    phi = (j + v) / PHI_BINS * 2 * np.pi
    r = np.sqrt(r2)
    return np.stack([(r * np.cos(phi)).ravel(), (r * np.sin(phi)).ravel()]), (i * PHI_BINS + j).ravel()


def fractal_phi_max(wi, xy, k):
    """phi_max of the fractal sampler for the zeta = k (wi + wo).xy of each point."""
    s = np.sqrt(max(0.0, 1.0 - wi[2] ** 2))
    f = k * np.sqrt((xy[0] + wi[0]) ** 2 + (xy[1] + wi[1]) ** 2)
    if s == 0.0:
        return np.full(f.shape, np.pi)
    with np.errstate(divide="ignore", invalid="ignore"):
        c = np.clip(((f / k) ** 2 + s * s - 1.0) / (2.0 * (f / k) * s), -1.0, 1.0)
    return np.where(f == 0.0, np.pi, np.arccos(c))


def expected(density, bins):
    e = np.bincount(bins, weights=density, minlength=R2_BINS * PHI_BINS)
    return e / e.sum()


def pvalue(observed, expected_frac, min_expected=5.0):
    """Pearson chi-square p-value; bins with fewer than min_expected expected samples are pooled."""
    from scipy.stats import chi2
    n = observed.sum()
    e = expected_frac * n
    keep = e >= min_expected
    o2 = np.append(observed[keep], observed[~keep].sum())
    e2 = np.append(e[keep], e[~keep].sum())
    if e2[-1] < min_expected:
        o2, e2 = o2[:-1], e2[:-1]
        # pooled low bins with no expectation must also have (almost) no samples
        assert observed[~keep].sum() <= max(5.0, 1e-4 * n), observed[~keep].sum()
    stat = float(((o2 - e2) ** 2 / e2).sum())
    return float(chi2.sf(stat, len(o2) - 1)), stat, len(o2) - 1


# ---- cases: (name, record factory, lobe family, density kind, wavenumber rule) -------------------
WAVELENGTH_NM = 550.0
K_550 = 2 * np.pi / (1e-3 * WAVELENGTH_NM)
K_MEAN = 2 * np.pi / 0.55     # FractalSurface's mean wavenumber (the opaque dielectric samples with it)


def cases():
    from pltfalcor_gb300 import materials as M
    au = (0, 1)   # Au (eta, k) in spectra.standard_profiles()
    return [
        ("dielectric_r0.45", lambda: M.dielectric(1, 0.45, ior=1.5), 0x02, "gauss", K_550),
        ("conductor_r0.35", lambda: M.conductor(1, 0.35, *au), 0x02, "fractal", K_550),
        ("conductor_r0.6_g2.5", lambda: M.conductor(1, 0.6, *au, gamma=2.5), 0x02, "fractal", K_550),
        ("opaque_dielectric_r0.4", lambda: M.opaque_dielectric(1, 0.4), 0x02, "fractal", K_MEAN),
        ("grated_conductor_r0.4", lambda: M.grated(1, True, 1.5, 0.1, roughness=0.4, ior_n_id=au[0], ior_k_id=au[1]), 0x02, "fractal",
         K_550),
        ("grated_opaque_r0.4", lambda: M.grated(1, False, 1.5, 0.1, roughness=0.4), 0x02, "fractal", K_MEAN),
        ("diffuse", lambda: M.diffuse(1, albedo=(0.7, 0.7, 0.7)), 0x01, "uniform", K_550),
    ]


WI = [(30.0, 20.0), (65.0, 200.0)]


def _batch(records, profiles, v, w, ops, frame=0):
    from pltfalcor_gb300 import workloads as W
    n = v.shape[1]
    rng = W.CounterRNG(99, n)
    wl = np.full(n, WAVELENGTH_NM, np.float32)
    stokes = np.zeros((4, n), np.float32)
    stokes[0] = 1.0
    coh = W._coherence(rng, wl)
    return W.Workload("chi2", n, 1, np.zeros(n, np.uint32), v.astype(np.float32).reshape(-1), w.astype(np.float32).reshape(-1),
                      None, wl, stokes.reshape(-1), coh.reshape(-1), records, profiles, ops, frame)


def sample_batch(records, profiles, wi, n, frame=0):
    v = np.repeat(wi[:, None], n, axis=1)
    return _batch(records, profiles, v, v, 0x4, frame)


def pdf_batch(records, profiles, wi):
    xy, bins = grid_points()
    z = np.sqrt(np.maximum(0.0, 1.0 - (xy ** 2).sum(axis=0))) * np.sign(wi[2])
    grid = np.vstack([xy, z])
    w = np.repeat(wi[:, None], grid.shape[1], axis=1)
    # pdf(sd.V = grid point, toLight = wi): the materials' pdf(wi, wo) with wi = toLight, wo = V
    return _batch(records, profiles, grid, w, 0x2), xy, bins


def run_case(run, records, profiles, family, kind, k, wi, n, frame=0):
    """`run(workload, ops)` returns the results dict (oracle.run or the library through the C ABI).
    Returns (p-value, statistic, dof, samples used)."""
    s = run(sample_batch(records, profiles, wi, n, frame), 0x4)
    wo = s["sample_wo"].reshape(3, -1).astype(np.float64)
    keep = (s["sample_valid"] == 1) & (s["sample_lobe"] == family)
    obs = histogram(wo[:2, keep])
    if kind == "uniform":
        _, bins = grid_points()
        dens = np.ones(len(bins))
    else:
        pw, xy, bins = pdf_batch(records, profiles, wi)
        dens = run(pw, 0x2)["pdf"].astype(np.float64)
        if kind == "fractal":
            dens = dens / fractal_phi_max(wi, xy, k)
    p, stat, dof = pvalue(obs, expected(dens, bins))
    return p, stat, dof, int(keep.sum())
