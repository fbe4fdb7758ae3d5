"""ORACLE -- test infrastructure only.  Freezes the algorithmic work per query of the benchmark
workload into profiles/op_counts_mixed_material.json, from the oracle's op-counting build (the
restated reference code run with a counting real type: FP32-pipe ops, special-function ops and
divides per query, material setup excluded, structural zeros of the sparse Mueller products not
counted).  bench.py reads the JSON (a data file) for the compute roofline.

Usage (from the repository root): python oracle/count_ops.py [n_sample]
"""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path[:0] = [ROOT, os.path.dirname(os.path.abspath(__file__))]

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from pltfalcor_gb300 import materials as M  # noqa: E402
from pltfalcor_gb300 import spectra  # noqa: E402
from pltfalcor_gb300 import workloads as W  # noqa: E402


def main():
    n = int(sys.argv[1]) if len(sys.argv) > 1 else 8 * 4096
    prof, _ = spectra.standard_profiles()
    wl = W.mixed_material_batch(n=1 << 22, profiles=prof).subset(np.arange(n))
    per = oracle.count_ops(wl, ops=0x7)
    tot = sum(v["count"] for v in per.values())
    mean = lambda k: sum(v[k] * v["count"] for v in per.values()) / tot
    out = {"workload": "mixed_material_batch (2^22, seed 1), first %d queries" % n, "ops": "eval+sample+pdf",
           "mean_fp_per_query": mean("fp"), "mean_sfu_per_query": mean("sfu"), "mean_div_per_query": mean("div"),
           "per_material": {M.TYPE_NAMES[t]: {k: float(v[k]) for k in ("fp", "sfu", "div")} | {"count": v["count"]} for t, v in per.items()},
           "counting": "FP32-pipe ops = add/sub/mul (+ fixed polynomial costs of exp/log/sin/cos/acos/atan2/pow); "
                       "SFU ops = sqrt, exp, log, sin, cos, acos, atan2, 2 per pow; divides counted separately"}
    dst = os.path.join(ROOT, "profiles", "op_counts_mixed_material.json")
    os.makedirs(os.path.dirname(dst), exist_ok=True)
    with open(dst, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps(out, indent=1))
    # the rough-dielectric eval + pdf batch (65,536 queries, seed 0), all of it
    wl0 = W.rough_dielectric_batch(n=65536, seed=0, profiles=prof)
    per0 = oracle.count_ops(wl0, ops=0x3)
    tot0 = sum(v["count"] for v in per0.values())
    mean0 = lambda k: sum(v[k] * v["count"] for v in per0.values()) / tot0
    out0 = {"workload": "rough_dielectric_batch (65,536 queries, seed 0)", "ops": "eval+pdf",
            "mean_fp_per_query": mean0("fp"), "mean_sfu_per_query": mean0("sfu"), "mean_div_per_query": mean0("div"),
            "counting": out["counting"]}
    with open(os.path.join(ROOT, "profiles", "op_counts_rough_dielectric.json"), "w") as f:
        json.dump(out0, f, indent=1)
    print(json.dumps(out0, indent=1))


if __name__ == "__main__":
    main()
