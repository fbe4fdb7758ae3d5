"""plt_bsdf_batch_noalloc, the batched BSDF entry point for callers that may not allocate device
memory (a per-frame render loop under a fixed memory budget, or a host application that owns every
device allocation).  It runs the same kernels as plt_bsdf_batch with its sorting scratch in a
fixed device array of the library, so its results must match plt_bsdf_batch's within the parity
tolerance -- on two calls in a row, since every call reuses (and must fully rewrite) that array.

This file is collected last on purpose; it passes alone in a fresh process and after the others.
"""
import ctypes as C

import numpy as np
import pytest

import parity
from pltfalcor_gb300 import capi
from pltfalcor_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.fail("CUDA device required for -m gpu tests")
    return torch


def test_noalloc_matches_batch_twice(torch_cuda, product_lib, profiles):
    from pltfalcor_gb300.bsdf import DeviceBatch, PLTContext
    lib = capi.load_library()
    ctx = PLTContext()
    ctx.set_spectral_profiles(profiles[0])
    ops = capi.OP_ALL
    # two different batches so the second call must overwrite what the first left in the array
    for n, hwss, seed in ((8 * 16384, 1, 1), (8 * 4096, 4, 3)):
        wl = W.mixed_material_batch(n=n, seed=seed, profiles=profiles[0], hwss=hwss)
        ctx.set_materials(wl.records)
        ref = DeviceBatch(wl)
        ctx.batch(ref.queries(), ref.results(ops), ops)
        assert ctx.check_status() == capi.PLT_OK
        expected = ref.fetch()
        for _ in range(2):
            b = DeviceBatch(wl)
            st = lib.plt_bsdf_batch_noalloc(ctx.handle, C.byref(b.queries()), C.byref(b.results(ops)), ops, None)
            assert st == capi.PLT_OK, capi.STATUS_NAMES.get(st, st)
            assert ctx.check_status() == capi.PLT_OK
            got = b.fetch()
            errs = parity.errors(got, expected, wl.n, wl.hwss, ops)
            assert not parity.check(errs), parity.summarize(errs)
    ctx.close()


def test_noalloc_rejects_oversized_batch(torch_cuda, product_lib):
    from pltfalcor_gb300.bsdf import PLTContext
    lib = capi.load_library()
    ctx = PLTContext()
    q = capi.BsdfQueries()
    q.n = capi.NOALLOC_MAX_QUERIES + 1
    q.hwss = 1
    r = capi.BsdfResults()
    assert lib.plt_bsdf_batch_noalloc(ctx.handle, C.byref(q), C.byref(r), capi.OP_EVAL, None) == capi.PLT_TOO_LARGE
    assert lib.plt_status_string(capi.PLT_TOO_LARGE).startswith(b"batch larger")
    ctx.close()
