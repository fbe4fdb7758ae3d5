"""Spectral tables: the conductor IORs (Au, Ag, Cu, Al) and the D65 emitter of the workloads.

The raw piecewise-linear samples live in data/spectral_tables.json (extracted from the reference's
Source/Tables by data/make_spectral_tables.py).  Profiles are built by the library's
plt_spectral_profile_from_samples, the restatement of SceneBuilder::addSpectralProfileFromMaterial
(IOR tables, no inverse CDF) and addSpectralProfileForEmitterType (emitters, with inverse CDF),
Source/Falcor/Scene/SceneBuilder.cpp:962-999.
"""
import ctypes as C
import json
import os

import numpy as np

from . import capi

DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "spectral_tables.json")
METALS = ["Au", "Ag", "Cu", "Al"]


def load_tables():
    with open(DATA) as f:
        return json.load(f)


def profile_from_samples(wavelengths, values, scale=1.0, compute_icdf=False, lib=None):
    lib = lib or capi.load_library()
    wl = np.ascontiguousarray(wavelengths, dtype=np.float32)
    v = np.ascontiguousarray(values, dtype=np.float32)
    out = capi.SpectralProfile()
    st = lib.plt_spectral_profile_from_samples(wl.ctypes.data_as(C.POINTER(C.c_float)), v.ctypes.data_as(C.POINTER(C.c_float)),
                                               len(wl), float(scale), int(compute_icdf), C.byref(out))
    capi.check(st, "plt_spectral_profile_from_samples")
    return out


def standard_profiles(lib=None):
    """Profiles in a fixed order: Au.eta, Au.k, Ag.eta, Ag.k, Cu.eta, Cu.k, Al.eta, Al.k, D65.
    Returns (ctypes array of SpectralProfile, {name: index})."""
    t = load_tables()
    names = [m + s for m in METALS for s in (".eta", ".k")] + ["D65"]
    arr = (capi.SpectralProfile * len(names))()
    for i, nm in enumerate(names):
        arr[i] = profile_from_samples(t[nm]["wavelength_nm"], t[nm]["value"], 1.0, nm == "D65", lib)
    return arr, {nm: i for i, nm in enumerate(names)}


def metal_ids(metal_index):
    """(n, k) profile ids of METALS[metal_index] in standard_profiles()."""
    return 2 * metal_index, 2 * metal_index + 1


def profile_from_spd(path, scale=1.0, compute_icdf=False, lib=None):
    """plt_spectral_profile_from_spd: a SpectralProfile built from a .spd table file."""
    import ctypes as C
    lib = lib or capi.load_library()
    out = capi.SpectralProfile()
    capi.check(lib.plt_spectral_profile_from_spd(os.fsencode(path), scale, 1 if compute_icdf else 0, C.byref(out)),
               "plt_spectral_profile_from_spd")
    return out


def profiles_from_material(tables_dir, name, lib=None):
    """plt_spectral_profiles_from_material: (eta, k) profiles of a named IOR table ("none": 1, 0)."""
    import ctypes as C
    lib = lib or capi.load_library()
    eta, k = capi.SpectralProfile(), capi.SpectralProfile()
    capi.check(lib.plt_spectral_profiles_from_material(os.fsencode(tables_dir), name.encode(), C.byref(eta), C.byref(k)),
               "plt_spectral_profiles_from_material")
    return eta, k


def profile_for_emitter_type(tables_dir, name, scale=1.0, lib=None):
    """plt_spectral_profile_for_emitter_type: the profile of a named emission table, scaled."""
    import ctypes as C
    lib = lib or capi.load_library()
    out = capi.SpectralProfile()
    capi.check(lib.plt_spectral_profile_for_emitter_type(os.fsencode(tables_dir), name.encode(), float(scale), C.byref(out)),
               "plt_spectral_profile_for_emitter_type")
    return out


def write_exr(path, rgba, half=False, lib=None):
    """plt_write_exr of a [height][width][4] float image (numpy or CPU tensor)."""
    import ctypes as C
    import numpy as np
    lib = lib or capi.load_library()
    a = np.ascontiguousarray(np.asarray(rgba, dtype=np.float32))
    h, w = a.shape[:2]
    capi.check(lib.plt_write_exr(os.fsencode(path), a.ctypes.data_as(C.POINTER(C.c_float)), w, h, 1 if half else 0), "plt_write_exr")
