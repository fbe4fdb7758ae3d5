"""Extracts the spectral data tables the PLT workloads use into spectral_tables.json.

Reads the reference repository's `.spd` files (Source/Tables/ior/{Au,Ag,Cu,Al}.{eta,k}.spd, from
the luxpop.com database, and Source/Tables/emission/D65.spd, the CIE D65 illuminant via lspdd.org)
and stores their (wavelength nm, value) pairs verbatim, with the source line, so that the GPU
host (which has no copy of the reference) can rebuild the SpectralProfiles with
plt_spectral_profile_from_samples.  The parser follows PiecewiseLinearSpectrum::fromFile
(Source/Falcor/Utils/Color/Spectrum.cpp:89-111): '#' lines and blank lines are skipped, parsing
stops at the first line that does not hold two numbers.

Usage: python pltfalcor_gb300/data/make_spectral_tables.py [reference_root]
"""
import json
import os
import sys

TABLES = {
    "Au.eta": "Source/Tables/ior/Au.eta.spd", "Au.k": "Source/Tables/ior/Au.k.spd",
    "Ag.eta": "Source/Tables/ior/Ag.eta.spd", "Ag.k": "Source/Tables/ior/Ag.k.spd",
    "Cu.eta": "Source/Tables/ior/Cu.eta.spd", "Cu.k": "Source/Tables/ior/Cu.k.spd",
    "Al.eta": "Source/Tables/ior/Al.eta.spd", "Al.k": "Source/Tables/ior/Al.k.spd",
    "D65": "Source/Tables/emission/D65.spd",
}


def parse_spd(path):
    wl, val, header = [], [], []
    with open(path, encoding="utf-8", errors="replace") as f:
        for line in f:
            s = line.strip()
            if not s:
                continue
            if s.startswith("#"):
                if len(header) < 3:
                    header.append(s)
                continue
            parts = s.split()
            try:
                a, b = float(parts[0]), float(parts[1])
            except (ValueError, IndexError):
                break
            wl.append(a)
            val.append(b)
    return wl, val, header


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python make_spectral_tables.py <reference source root (the directory holding Source/Tables)>")
    root = sys.argv[1]
    out = {}
    for name, rel in TABLES.items():
        wl, val, header = parse_spd(os.path.join(root, rel))
        out[name] = {"source": rel, "header": header, "wavelength_nm": wl, "value": val}
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "spectral_tables.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", dst, {k: len(v["value"]) for k, v in out.items()})


if __name__ == "__main__":
    main()
