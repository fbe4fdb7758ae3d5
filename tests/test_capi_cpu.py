"""C-ABI library tests that need no GPU: it loads, exports every declared symbol, and its host-only
entry points (options, status strings, spectral profile builder) behave."""
import ctypes as C
import os
import re

import numpy as np

from pltfalcor_gb300 import capi, spectra

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "plt_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:[a-z_0-9]+\s*\*?\s+)+\*?(plt_[a-z_0-9]+)\s*\(", src, re.M)))


def test_exports_every_declared_symbol(product_lib):
    decl = declared_symbols()
    assert len(decl) >= 15
    assert set(decl) == set(capi.EXPORTED_SYMBOLS)
    for s in decl:
        assert hasattr(product_lib, s), s


def test_abi_version_and_status_strings(product_lib):
    assert product_lib.plt_abi_version() == 5
    assert product_lib.plt_status_string(0) == b"ok"
    assert product_lib.plt_status_string(7) == b"bad material"


def test_options_default_matches_pltpt(product_lib):
    o = capi.Options()
    assert product_lib.plt_options_default(C.byref(o)) == 0
    # PLTPT.h:74-108 defaults
    assert (o.max_bounces, o.tile_size, o.hwss, o.mnee_max_occluders, o.mnee_max_iterations) == (32, 512, 4, 2, 60)
    assert o.emissive_sampler == 2   # EmissiveLightSamplerType::Power (PLTPT.h:99)
    assert abs(o.mnee_solver_threshold - 5e-5) < 1e-9 and abs(o.sourcing_max_beam_omega - 0.025) < 1e-9
    # every key of PLTPT::parseDictionary (PLTPT.cpp:147-175) has a field with the PLTPT.h default
    keys = {"maxBounces": o.max_bounces, "tileSize": o.tile_size, "debugView": o.debug_view,
            "debugViewIntensity": o.debug_view_intensity, "sourcingAreaFromEmissiveGeometry": o.sourcing_area_from_emissive_geometry,
            "sourcingMaxBeamOmega": o.sourcing_max_beam_omega, "sampleGenerator": o.sample_generator, "HWSS": o.hwss,
            "HWSSDoMIS": o.hwss_do_mis, "useDirectLights": o.use_direct_light, "useEnvLights": o.use_env_light,
            "useEmissiveLights": o.use_emissive_lights, "useAnalyticLights": o.use_analytic_lights, "alphaMasking": o.alpha_masking,
            "doNEE": o.do_nee, "NEEUsePerTileSG": o.nee_use_per_tile_sg, "doMIS": o.do_mis, "emissiveSampler": o.emissive_sampler,
            "doRussianRoulette": o.do_russian_roulette, "doImportanceSampleEmitters": o.do_importance_sample_emitters,
            "doMNEE": o.do_mnee, "MNEEMaxOccluders": o.mnee_max_occluders, "MNEEMaxIterations": o.mnee_max_iterations}
    assert keys["debugView"] == capi.DEBUG_VIEW_NONE and keys["debugViewIntensity"] == 1.0
    assert keys["sampleGenerator"] == capi.SAMPLE_GENERATOR_UNIFORM   # SAMPLE_GENERATOR_DEFAULT
    assert keys["alphaMasking"] == 1 and keys["sourcingAreaFromEmissiveGeometry"] == 1.0
    assert all(keys[k] == 1 for k in ("HWSSDoMIS", "useDirectLights", "useEnvLights", "useEmissiveLights", "useAnalyticLights",
                                      "doNEE", "doMIS", "doRussianRoulette", "doImportanceSampleEmitters", "doMNEE"))
    assert keys["NEEUsePerTileSG"] == 0


def test_spectral_profile_builder_matches_oracle(product_lib, oracle_lib):
    t = spectra.load_tables()
    for name in ("Au.eta", "Cu.k", "Al.eta", "D65"):
        wl = np.ascontiguousarray(t[name]["wavelength_nm"], np.float32)
        v = np.ascontiguousarray(t[name]["value"], np.float32)
        icdf = int(name == "D65")
        a = capi.SpectralProfile()
        b = capi.SpectralProfile()
        fp = C.POINTER(C.c_float)
        assert product_lib.plt_spectral_profile_from_samples(wl.ctypes.data_as(fp), v.ctypes.data_as(fp), len(wl), 1.0, icdf, C.byref(a)) == 0
        assert oracle_lib.plto_spectral_profile_from_samples(wl.ctypes.data_as(fp), v.ctypes.data_as(fp), len(wl), 1.0, icdf, C.byref(b)) == 0
        assert a.bins == b.bins and 0 < a.bins <= 128
        assert a.min_wavelength == max(380.0, float(wl[0])) and a.max_wavelength == min(720.0, float(wl[-1]))
        assert list(a.pdf) == list(b.pdf) and list(a.icdf) == list(b.icdf) and a.intensity == b.intensity
        if icdf:
            assert abs(sum(a.pdf[: a.bins]) - 1.0) < 1e-4
            assert all(np.diff(np.asarray(a.icdf[: a.bins])) >= -1e-7)


def test_spectral_profile_rejects_bad_input(product_lib):
    fp = C.POINTER(C.c_float)
    wl = np.float32([500, 400, 600])
    v = np.float32([1, 2, 3])
    out = capi.SpectralProfile()
    assert product_lib.plt_spectral_profile_from_samples(wl.ctypes.data_as(fp), v.ctypes.data_as(fp), 3, 1.0, 0, C.byref(out)) == capi.PLT_INVALID_ARG
    assert product_lib.plt_spectral_profile_from_samples(None, None, 0, 1.0, 0, C.byref(out)) == capi.PLT_INVALID_ARG
