"""Builds libplt_gb300.so in-tree (pltfalcor_gb300/_build/) for sm_103a.

CUDA sources go through nvcc with `-gencode arch=compute_103a,code=sm_103a -lineinfo`; host C++
sources through g++ with FP contraction off (the host evaluates material constants with the same
float expressions as the shader source).  Translation units compile in parallel.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libplt_gb300.so")

CU_SOURCES = ["plt_bsdf_h1.cu", "plt_bsdf_h2.cu", "plt_bsdf_h3.cu", "plt_bsdf_h4.cu", "plt_bsdf_h8.cu", "plt_trace.cu", "plt_noalloc.cu",
              "plt_pt.cu", "plt_pt_h1.cu", "plt_pt_h2.cu", "plt_pt_h3.cu", "plt_pt_h4.cu", "plt_pt_h8.cu", "plt_mlp.cu",
              "plt_envmap.cu"]
CPP_SOURCES = ["plt_capi.cpp", "plt_materials.cpp", "plt_bsdf_dispatch.cpp", "plt_bvh.cpp", "plt_render.cpp", "plt_proposal.cpp",
               "plt_scenes.cpp", "plt_io.cpp", "plt_host_batch.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Single-precision division and square root use the SFU approximations (<= 2 ulp, the accuracy
# class D3D allows the reference shaders).  The BSDF batch units also flush subnormals to zero and
# take the SFU approximations of sin, cos, exp, log and exp2 (--use_fast_math), as D3D and Vulkan
# shaders do by default: FP32 results below 1.2e-38 carry no radiance the parity bound can see (the
# interference cross term, the one place a product of two small intensities becomes subnormal, is
# computed in a form that does not underflow), and the approximations' errors (absolute 2^-20.5 for
# sin and cos up to 100 pi, relative ~2^-21 for exp2) are inside D3D's bounds for the shaders'
# intrinsics.  Divisions and square roots that must be exact stay explicitly rounded intrinsics.
# The render and traversal units keep subnormals and the accurate functions: the ray/triangle test
# is bit-exact against the oracle.
CU_FLAGS = ["-prec-div=false", "-prec-sqrt=false"]
BSDF_UNITS = {"plt_bsdf_h1.cu", "plt_bsdf_h2.cu", "plt_bsdf_h3.cu", "plt_bsdf_h4.cu", "plt_bsdf_h8.cu", "plt_noalloc.cu"}


def unit_flags(source):
    """nvcc flags specific to one translation unit (see above)."""
    return ["-ftz=true", "--use_fast_math"] if os.path.basename(source) in BSDF_UNITS else ["-ftz=false"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found")
    return cand


def _cuda_home():
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False, ptxas_verbose=False, defines=(), build_dir=None, nvcc_flags=()):
    """Compiles the library.  `defines` (e.g. ["PLT_SHADE_MIN_BLOCKS=6"]), `nvcc_flags` and
    `build_dir` build a tuning variant elsewhere; the default build is
    pltfalcor_gb300/_build/libplt_gb300.so."""
    bdir = build_dir or BUILD
    lib = os.path.join(bdir, "libplt_gb300.so")
    os.makedirs(bdir, exist_ok=True)
    nvcc = _nvcc()
    dflags = ["-D" + d for d in defines]
    cuflags = list(CU_FLAGS) + list(nvcc_flags)
    inc = os.path.join(_cuda_home(), "include")
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "plt_gb300.h"))
    jobs = []
    objs = []
    for s in CU_SOURCES:
        src, obj = os.path.join(CSRC, s), os.path.join(bdir, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            cmd = [nvcc, *ARCH, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "--expt-relaxed-constexpr", *unit_flags(s), *cuflags, *dflags, "-c", src, "-o", obj]
            if ptxas_verbose:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for s in CPP_SOURCES:
        src, obj = os.path.join(CSRC, s), os.path.join(bdir, s + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-I", inc,
                         *dflags, "-c", src, "-o", obj])
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    if force or _stale(lib, objs):
        _run([nvcc, *ARCH, "-shared", "-o", lib, *objs, "-lcudart"])
    return lib


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv, ptxas_verbose="-v" in sys.argv))
