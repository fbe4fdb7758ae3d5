"""Regenerates the oracle fixtures in tests/golden/ (FP32 and FP64 oracle outputs of the query sets
in tests/golden_cases.py).  The inputs are regenerated from their seeds; only outputs are stored.

Usage (from the repository root): python tests/golden/make_golden.py
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]

import numpy as np  # noqa: E402

import golden_cases  # noqa: E402
import oracle  # noqa: E402
from pltfalcor_gb300 import build, spectra  # noqa: E402


def main():
    build.build()
    oracle.build()
    prof, _ = spectra.standard_profiles()
    for name, wl in golden_cases.cases(prof).items():
        out = {}
        # FP32, FP64 and FP32 with random rounding (seeds 1 and 2)
        for tag, prec, seed in (("fp32", 32, 1), ("fp64", 64, 1), ("rr", 16, 1), ("rr2", 16, 2)):
            res = oracle.run(wl, ops=0xF, precision=prec, sr_seed=seed)
            for k, v in res.items():
                out["%s_%s" % (k, tag)] = v
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), name + ".npz")
        np.savez_compressed(path, **out)
        print("wrote", path, wl.n)


if __name__ == "__main__":
    main()
