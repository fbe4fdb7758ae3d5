"""Build flags per translation unit (pltfalcor_gb300/build.py): which units take the shader
intrinsics' arithmetic (flushed subnormals, SFU approximations of the transcendental functions) and
which keep the accurate functions, and that every CUDA unit is built for sm_103a only."""
import os

from pltfalcor_gb300 import build


def test_fast_math_only_in_the_bsdf_batch_units():
    fast = {"plt_bsdf_h1.cu", "plt_bsdf_h2.cu", "plt_bsdf_h3.cu", "plt_bsdf_h4.cu", "plt_bsdf_h8.cu", "plt_noalloc.cu"}
    for src in build.CU_SOURCES:
        flags = build.unit_flags(src)
        if src in fast:
            assert flags == ["-ftz=true", "--use_fast_math"], src
        else:
            # traversal hits are bit-exact against the oracle; the render units' manifold walks
            # follow the oracle's success and failure with the accurate functions
            assert flags == ["-ftz=false"], src
    assert fast <= set(build.CU_SOURCES)
    # the batch kernels reached through plt_bsdf_batch and plt_bsdf_batch_noalloc give the same bits
    assert build.unit_flags("plt_noalloc.cu") == build.unit_flags("plt_bsdf_h1.cu")


def test_single_architecture_and_division_flags():
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert "-prec-div=false" in build.CU_FLAGS and "-prec-sqrt=false" in build.CU_FLAGS
    for src in build.CU_SOURCES + build.CPP_SOURCES:
        assert os.path.exists(os.path.join(build.CSRC, src)), src
