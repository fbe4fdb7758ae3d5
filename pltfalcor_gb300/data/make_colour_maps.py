"""Extracts the magma and inferno colour-map tables (256 RGB entries each) that the PLTPT debug
views colour-code with (Source/RenderPasses/PLTPT/ColourCoding.slang, ccMagma / ccInferno; the
tables are the published matplotlib colour maps) into csrc/plt_colour_maps.h, shared by the library
and the oracle.

    python make_colour_maps.py <reference source root (the directory holding Source/)>
"""
import os
import re
import sys


def table(text, name):
    m = re.search(r"float3\s+%s\s*\(float val\)\s*\{.*?data\[bins\]\s*=\s*\{(.*?)\};" % name, text, re.S)
    if not m:
        raise SystemExit("table %s not found" % name)
    rows = re.findall(r"\{\s*([-0-9.eE+]+)\s*,\s*([-0-9.eE+]+)\s*,\s*([-0-9.eE+]+)\s*\}", m.group(1))
    if len(rows) != 256:
        raise SystemExit("table %s has %d rows" % (name, len(rows)))
    return rows


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python make_colour_maps.py <reference source root (the directory holding Source/)>")
    src = os.path.join(sys.argv[1], "Source", "RenderPasses", "PLTPT", "ColourCoding.slang")
    with open(src) as f:
        text = f.read()
    here = os.path.dirname(os.path.abspath(__file__))
    dst = os.path.join(os.path.dirname(here), "csrc", "plt_colour_maps.h")
    out = ["// Generated by pltfalcor_gb300/data/make_colour_maps.py: the magma and inferno colour maps (256",
           "// RGB entries, the published matplotlib tables) that the PLTPT debug views colour-code scalars",
           "// with.  Included by the render pass and by the oracle.",
           "// Device code defines PLT_COLOUR_MAP_STORAGE (e.g. as static __constant__ const) before including it.",
           "#pragma once", "",
           "#ifndef PLT_COLOUR_MAP_STORAGE",
           "#define PLT_COLOUR_MAP_STORAGE static const",
           "#endif", ""]
    for cname, sname in (("kMagma", "ccMagma"), ("kInferno", "ccInferno")):
        rows = table(text, sname)
        out.append("PLT_COLOUR_MAP_STORAGE float %s[256][3] = {" % cname)
        for r in rows:
            out.append("    {%sf, %sf, %sf}," % r)
        out.append("};")
        out.append("")
    with open(dst, "w") as f:
        f.write("\n".join(out))
    print("wrote", dst)


if __name__ == "__main__":
    main()
