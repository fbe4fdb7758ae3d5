"""pltfalcor_gb300 -- GB300-native (sm_103a) PLT generalized-ray BSDF hot path of PLTFalcor.

The product is libplt_gb300.so (C ABI in include/plt_gb300.h, CUDA kernels in csrc/); this
package holds its Python mirror: ctypes bindings (capi), material packing (materials), spectral
tables (spectra), seeded workloads (workloads) and the batched IMaterialInstance API (bsdf).
"""
from . import capi, materials, spectra, workloads  # noqa: F401

__all__ = ["capi", "materials", "spectra", "workloads", "bsdf", "build"]
