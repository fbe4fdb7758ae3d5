"""Comparison helpers for GPU-vs-oracle parity (imported by the tests and by smoke()).

Tolerance (FP32 GPU vs the FP32 oracle, the reference arithmetic type), per query:

    err(gpu, oracle32) <= max(TOL, K * cond),   TOL = 1e-4, K = 10,
    cond = max(err(oracle32, oracle64), err(oracle32, oracle32 with random rounding, seeds 1 and 2))

where err is the relative error below.  `cond` is the conditioning allowance: where the FP32
reference arithmetic is itself ill-conditioned (1 - alpha with alpha -> 1 on smooth surfaces,
resonant multilayer recursions with phases of ~100 rad, BesselJ at grazing incidence, refraction
out of a coat at the critical angle, near-zero interference minima), its distance from the FP64
oracle and its spread under random rounding (Monte Carlo arithmetic: every FP32 operation rounded
up or down at random) bound how closely any second FP32 evaluation (FMA contraction, CUDA vs libm
special functions) can agree with it.  Queries inside the plain 1e-4 bound need neither.

Relative errors:
  - Stokes: per query and wavelength max_c |g_c - o_c| / |o_0| (components are bounded by S0);
  - pdf, lambdaPdf, sample pdf and weight: |g - o| / |o|;
  - coherence D: |g - o| / (|o_D0| + |o_D2|);
  - sample direction: |g - o|_inf (unit vectors);
  - discrete outputs (sampled lobe, validity): bit-exact.  Independent roundings can flip a
    discrete choice (u < pdf, a lobe cdf) when u lies within an ulp of the threshold; such queries
    are excluded from the continuous sample checks and counted.
The pass criterion allows at most `max_bad_frac` (default 1e-3) of queries outside the bound per
output and material.
"""
import numpy as np

TOL = 1e-4
K_COND = 10.0


def rel(a, b, denom):
    d = np.abs(a.astype(np.float64) - b.astype(np.float64))
    return np.where(d == 0, 0.0, d / np.maximum(denom, 1e-30))


def errors(a, ref, n, hwss, ops):
    """Per-output arrays of relative errors of `a` against `ref` (one value per query)."""
    out = {}
    if ops & 1:
        g = a["stokes"].reshape(4, hwss, n)
        o = ref["stokes"].reshape(4, hwss, n)
        den = np.abs(o[0].astype(np.float64))
        out["stokes"] = np.max(np.max(rel(g, o, den[None]), axis=0), axis=0)
        gc = a["coherence"].reshape(4, n)
        oc = ref["coherence"].reshape(4, n)
        dd = np.abs(oc[0].astype(np.float64)) + np.abs(oc[2].astype(np.float64))
        out["coherence"] = np.max(rel(gc[:3], oc[:3], dd[None]), axis=0)
    if ops & 2:
        out["pdf"] = rel(a["pdf"], ref["pdf"], np.abs(ref["pdf"].astype(np.float64)))
    if ops & 8:
        g = a["lambda_pdf"].reshape(hwss, n)
        o = ref["lambda_pdf"].reshape(hwss, n)
        out["lambda_pdf"] = np.max(rel(g, o, np.abs(o.astype(np.float64))), axis=0)
    if ops & 4:
        same = (a["sample_lobe"] == ref["sample_lobe"]) & (a["sample_valid"] == ref["sample_valid"])
        out["sample_discrete_mismatch"] = ~same
        gw = a["sample_wo"].reshape(3, n)
        ow = ref["sample_wo"].reshape(3, n)
        out["sample_wo"] = np.where(same, np.max(np.abs(gw.astype(np.float64) - ow), axis=0), 0.0)
        out["sample_pdf"] = np.where(same, rel(a["sample_pdf"], ref["sample_pdf"], np.abs(ref["sample_pdf"].astype(np.float64))), 0.0)
        out["sample_weight"] = np.where(same, rel(a["sample_weight"], ref["sample_weight"], np.abs(ref["sample_weight"].astype(np.float64))), 0.0)
    for k, v in out.items():
        if v.dtype != bool:
            out[k] = np.where(np.isnan(v), np.inf, v)
    return out


def compare(gpu, ora32, n, hwss, ops, ora64=None, ora32_rr=None):
    """Errors of the GPU against the FP32 oracle, with the per-query allowance derived from the
    FP32 oracle's own error against the FP64 oracle and its random-rounding spread (when given;
    `ora32_rr` may be one run or a list of runs with different seeds)."""
    e = errors(gpu, ora32, n, hwss, ops)
    rr = ora32_rr if isinstance(ora32_rr, (list, tuple)) else [ora32_rr]
    refs = [r for r in [ora64] + rr if r is not None]
    if refs:
        cs = [errors(ora32, r, n, hwss, ops) for r in refs]
        for k in list(e):
            if e[k].dtype != bool:
                e[k + "@allow"] = K_COND * np.maximum.reduce([c[k] for c in cs])
    return e


def bad_mask(errs, key, tol=TOL):
    v = errs[key]
    if v.dtype == bool:
        return v
    allow = errs.get(key + "@allow")
    bound = tol if allow is None else np.maximum(tol, allow)
    return v > bound


def summarize(errs, tol=TOL, sel=None):
    s = {}
    for k, v in errs.items():
        if k.endswith("@allow"):
            continue
        vv = v if sel is None else v[sel]
        if vv.size == 0:
            continue
        if v.dtype == bool:
            s[k] = {"frac": float(vv.mean())}
        else:
            b = bad_mask(errs, k, tol)
            b = b if sel is None else b[sel]
            s[k] = {"max": float(vv.max()), "p99": float(np.quantile(vv, 0.99)), "p50": float(np.quantile(vv, 0.5)),
                    "frac_above_tol": float((vv > tol).mean()), "frac_bad": float(b.mean())}
    return s


def check(errs, tol=TOL, max_bad_frac=1e-3, sel=None):
    """Returns a list of failure strings (empty if parity holds)."""
    fails = []
    for k, st in summarize(errs, tol, sel).items():
        if "frac" in st:
            if st["frac"] > max_bad_frac:
                fails.append("%s mismatch fraction %.3g > %.3g" % (k, st["frac"], max_bad_frac))
        elif st["frac_bad"] > max_bad_frac:
            fails.append("%s: %.3g of queries outside the bound (%.3g above %.0e, max %.3g)" %
                         (k, st["frac_bad"], st["frac_above_tol"], tol, st["max"]))
    return fails
