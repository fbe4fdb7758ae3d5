"""Comparison helpers for GPU-vs-oracle parity (imported by the tests and by smoke()).

Tolerances (FP32 GPU vs FP32 oracle, the reference arithmetic type):
  - Stokes outputs: per query and wavelength, max_c |g_c - o_c| / max(|o_0|, 1e-30) <= 1e-4
    (Stokes components are bounded by S0, so S0 normalises all four);
  - pdf, lambdaPdf, sample pdf and weight: |g - o| / max(|o|, 1e-30) <= 1e-4;
  - coherence D: |g - o| / max(|o_D0| + |o_D2|, 1e-30) <= 1e-4;
  - sample direction: |g - o|_inf <= 1e-4 (unit vectors);
  - discrete outputs (sampled lobe, validity) bit-exact.
Independent FP32 roundings (FMA contraction, CUDA vs libm special functions) can flip a discrete
choice (u < pdf, lobe cdf) when u lies within an ulp of the threshold, and can amplify rounding in
cancellations; a query whose discrete sample outcome differs is excluded from the continuous
sample checks and counted, and the pass criterion allows at most `max_bad_frac` of queries out of
tolerance per output.
"""
import numpy as np

TOL = 1e-4


def rel(a, b, denom):
    return np.abs(a.astype(np.float64) - b.astype(np.float64)) / np.maximum(denom, 1e-30)


def compare(gpu, ora, n, hwss, ops, tol=TOL):
    """Per-output arrays of relative errors (one value per query) plus discrete mismatch masks."""
    out = {}
    if ops & 1:
        g = gpu["stokes"].reshape(4, hwss, n)
        o = ora["stokes"].reshape(4, hwss, n)
        den = np.abs(o[0].astype(np.float64))
        e = np.max(rel(g, o, den[None]), axis=0)  # (hwss, n)
        # both zero -> 0 error (rel() gives 0/1e-30 = 0)
        out["stokes"] = np.max(e, axis=0)
        gc = gpu["coherence"].reshape(4, n)
        oc = ora["coherence"].reshape(4, n)
        dd = np.abs(oc[0].astype(np.float64)) + np.abs(oc[2].astype(np.float64))
        out["coherence"] = np.max(rel(gc[:3], oc[:3], dd[None]), axis=0)
    if ops & 2:
        out["pdf"] = rel(gpu["pdf"], ora["pdf"], np.abs(ora["pdf"].astype(np.float64)))
    if ops & 8:
        g = gpu["lambda_pdf"].reshape(hwss, n)
        o = ora["lambda_pdf"].reshape(hwss, n)
        out["lambda_pdf"] = np.max(rel(g, o, np.abs(o.astype(np.float64))), axis=0)
    if ops & 4:
        same = (gpu["sample_lobe"] == ora["sample_lobe"]) & (gpu["sample_valid"] == ora["sample_valid"])
        out["sample_discrete_mismatch"] = ~same
        gw = gpu["sample_wo"].reshape(3, n)
        ow = ora["sample_wo"].reshape(3, n)
        ewo = np.max(np.abs(gw.astype(np.float64) - ow), axis=0)
        out["sample_wo"] = np.where(same, ewo, 0.0)
        out["sample_pdf"] = np.where(same, rel(gpu["sample_pdf"], ora["sample_pdf"], np.abs(ora["sample_pdf"].astype(np.float64))), 0.0)
        out["sample_weight"] = np.where(same, rel(gpu["sample_weight"], ora["sample_weight"], np.abs(ora["sample_weight"].astype(np.float64))), 0.0)
    return out


def summarize(errs, tol=TOL, sel=None):
    s = {}
    for k, v in errs.items():
        vv = v if sel is None else v[sel]
        if vv.size == 0:
            continue
        if v.dtype == bool:
            s[k] = {"frac": float(vv.mean())}
        else:
            vv = np.where(np.isnan(vv), np.inf, vv)
            s[k] = {"max": float(vv.max()), "p99": float(np.quantile(vv, 0.99)), "frac_bad": float((vv > tol).mean())}
    return s


def check(errs, tol=TOL, max_bad_frac=1e-3, sel=None):
    """Returns a list of failure strings (empty if parity holds)."""
    fails = []
    for k, st in summarize(errs, tol, sel).items():
        if "frac" in st:
            if st["frac"] > max_bad_frac:
                fails.append("%s mismatch fraction %.3g > %.3g" % (k, st["frac"], max_bad_frac))
        elif st["frac_bad"] > max_bad_frac:
            fails.append("%s: %.3g of queries above %.0e (max %.3g)" % (k, st["frac_bad"], tol, st["max"]))
    return fails
