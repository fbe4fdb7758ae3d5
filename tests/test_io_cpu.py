"""Host-side I/O of the library (no GPU): the .spd spectral-table loader against the sample-based
profile builder, and the OpenEXR writer read back by an independent minimal EXR parser."""
import json
import os
import struct

import numpy as np
import pytest

from pltfalcor_gb300 import capi, spectra


def _profile_bytes(p):
    import ctypes as C
    return bytes(C.string_at(C.addressof(p), C.sizeof(p)))


def test_spd_loader_equals_sample_builder(product_lib, tmp_path):
    tables = spectra.load_tables()
    for name in ("D65", "Au.eta", "Cu.k"):
        wl, val = np.asarray(tables[name]["wavelength_nm"], np.float32), np.asarray(tables[name]["value"], np.float32)
        path = tmp_path / ("%s.spd" % name)
        with open(path, "w") as f:
            f.write("# %s\n# wavelength value\n\n" % name)
            for a, b in zip(wl, val):
                f.write("%r %r\n" % (float(a), float(b)))
            f.write("end of data\n7 8\n")     # reading stops at the first line without two numbers
        for icdf in (False, True):
            a = spectra.profile_from_spd(str(path), 2.0, icdf)
            b = spectra.profile_from_samples(wl, val, 2.0, icdf)
            assert _profile_bytes(a) == _profile_bytes(b), name


def test_spd_loader_rejects_missing_and_empty(product_lib, tmp_path):
    lib = capi.load_library()
    out = capi.SpectralProfile()
    import ctypes as C
    assert lib.plt_spectral_profile_from_spd(b"/nonexistent/x.spd", 1.0, 0, C.byref(out)) == capi.PLT_INVALID_ARG
    p = tmp_path / "empty.spd"
    p.write_text("# nothing\n")
    assert lib.plt_spectral_profile_from_spd(os.fsencode(str(p)), 1.0, 0, C.byref(out)) == capi.PLT_INVALID_ARG


def test_named_table_lookups(product_lib, tmp_path):
    """plt_spectral_profiles_from_material / plt_spectral_profile_for_emitter_type read the
    reference's Tables layout (ior/<name>.eta.spd + .k.spd without inverse CDFs, emission/<name>.spd
    scaled with one) and equal the direct .spd loads; "none" is n = 1, k = 0 in one bin."""
    tables = spectra.load_tables()
    (tmp_path / "ior").mkdir()
    (tmp_path / "emission").mkdir()

    def write(path, name):
        wl, val = tables[name]["wavelength_nm"], tables[name]["value"]
        with open(path, "w") as f:
            for a_, b_ in zip(wl, val):
                f.write("%r %r\n" % (float(a_), float(b_)))

    write(tmp_path / "ior" / "Au.eta.spd", "Au.eta")
    write(tmp_path / "ior" / "Au.k.spd", "Au.k")
    write(tmp_path / "emission" / "d65.spd", "D65")
    eta, k = spectra.profiles_from_material(str(tmp_path), "Au")
    assert _profile_bytes(eta) == _profile_bytes(spectra.profile_from_spd(str(tmp_path / "ior" / "Au.eta.spd"), 1.0, False))
    assert _profile_bytes(k) == _profile_bytes(spectra.profile_from_spd(str(tmp_path / "ior" / "Au.k.spd"), 1.0, False))
    em = spectra.profile_for_emitter_type(str(tmp_path), "d65", 3.0)
    assert _profile_bytes(em) == _profile_bytes(spectra.profile_from_spd(str(tmp_path / "emission" / "d65.spd"), 3.0, True))
    n1, k0 = spectra.profiles_from_material(str(tmp_path), "none")
    assert n1.bins == 1 and n1.pdf[0] == 1.0 and k0.bins == 1 and k0.pdf[0] == 0.0
    with pytest.raises(RuntimeError):
        spectra.profiles_from_material(str(tmp_path), "Ag")
    with pytest.raises(RuntimeError):
        spectra.profile_for_emitter_type(str(tmp_path), "missing")


def _read_exr(path):
    """Minimal reader of uncompressed single-part scanline OpenEXR files."""
    data = open(path, "rb").read()
    assert struct.unpack_from("<I", data, 0)[0] == 20000630
    pos, attrs = 8, {}
    while data[pos] != 0:
        name_end = data.index(b"\0", pos)
        name = data[pos:name_end].decode()
        type_end = data.index(b"\0", name_end + 1)
        typ = data[name_end + 1:type_end].decode()
        size = struct.unpack_from("<i", data, type_end + 1)[0]
        attrs[name] = (typ, data[type_end + 5:type_end + 5 + size])
        pos = type_end + 5 + size
    pos += 1
    chl, chans, cpos = attrs["channels"][1], [], 0
    while chl[cpos] != 0:
        e = chl.index(b"\0", cpos)
        chans.append((chl[cpos:e].decode(), struct.unpack_from("<i", chl, e + 1)[0]))
        cpos = e + 1 + 16
    assert attrs["compression"][1] == b"\0"
    x0, y0, x1, y1 = struct.unpack("<4i", attrs["dataWindow"][1])
    w, h = x1 - x0 + 1, y1 - y0 + 1
    offsets = struct.unpack_from("<%dQ" % h, data, pos)
    img = {c: np.zeros((h, w), np.float32) for c, _ in chans}
    for y in range(h):
        o = offsets[y]
        yy, size = struct.unpack_from("<ii", data, o)
        o += 8
        for c, t in chans:
            dt = np.float16 if t == 1 else np.float32
            n = w * np.dtype(dt).itemsize
            img[c][yy] = np.frombuffer(data, dt, w, o).astype(np.float32)
            o += n
    return np.stack([img["R"], img["G"], img["B"], img["A"]], axis=-1)


@pytest.mark.parametrize("half", [False, True])
def test_exr_round_trip(product_lib, tmp_path, half):
    rng = np.random.default_rng(5)
    img = rng.uniform(0, 50, (7, 13, 4)).astype(np.float32)
    img[..., 3] = 1.0
    img[0, 0, 0] = 65504.0 if half else 3.0e38
    path = str(tmp_path / "img.exr")
    spectra.write_exr(path, img, half=half)
    back = _read_exr(path)
    ref = img.astype(np.float16).astype(np.float32) if half else img
    assert np.array_equal(back, ref)
