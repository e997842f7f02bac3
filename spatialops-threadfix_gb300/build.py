"""Build recipe for libnebo_gb300.so (sm_103a only) and the C++ test programs.

    python spatialops-threadfix_gb300/build.py

compiles every csrc/*.cu in parallel with
    nvcc -gencode arch=compute_103a,code=sm_103a -O3 -lineinfo -std=c++17 -Xcompiler -fPIC
and links them (static CUDA runtime) into spatialops-threadfix_gb300/_build/libnebo_gb300.so.
Objects are rebuilt only when a source or header is newer.  nvcc cross-compiles, so this runs
on a host without a GPU too.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(REPO, "include")
LIB = os.path.join(BUILD, "libnebo_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
                     "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _headers():
    return glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, obj, extra=(), resources=False):
    cmd = [nvcc(), *NVCC_FLAGS, *extra, *(["-Xptxas", "-v"] if resources else []), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stderr}")
    if resources:  # ptxas's register / shared memory / spill report per kernel, beside the object
        with open(obj + ".resources.txt", "w") as f:
            f.write(r.stderr)
    return obj


TESTS_CPP = os.path.join(REPO, "tests", "cpp")
TESTS_BUILD = os.path.join(TESTS_CPP, "_build")
# C++ programs written against the drop-in headers (include/spatialops): name -> (source, flags)
PROGRAMS = {
    # exact: no contraction anywhere, user functors (apply_pointwise) included
    "catalog_gpu_exact": ("catalog_gpu.cu", ["-DNEBO_EXACT_ARITHMETIC", "--fmad=false"]),
    "catalog_gpu_fast": ("catalog_gpu.cu", []),
    # particle <-> cell scenes (tests/cpp/particles_scene.h) on the drop-in headers
    "particles_gpu": ("particles_gpu.cu", []),
    # `<<=` timing against the hand-fused kernels: the default lowering, the reference GPU
    # kernel's design (one thread per column, CUDA's exp/sin), and the tiled lowering with CUDA's
    # exp/sin
    "assign_timing": ("assign_timing.cu", []),
    "assign_timing_untiled": ("assign_timing.cu", ["-DNEBO_UNTILED", "-DNEBO_CUDA_LIBM"]),
    "assign_timing_libm": ("assign_timing.cu", ["-DNEBO_CUDA_LIBM"]),
    # `<<=` on FP32 fields against FP64 (the lowering passes on float)
    "float_assign": ("float_assign.cu", []),
    # the heat and transport configurations written in Nebo (golden checks, and the transport
    # timed against the hand kernel)
    "configs_dropin": ("configs_dropin.cu", []),
}


def _dropin_headers():
    return glob.glob(os.path.join(INCLUDE, "spatialops", "**", "*.h"), recursive=True) + \
        glob.glob(os.path.join(TESTS_CPP, "*.h")) + glob.glob(os.path.join(TESTS_CPP, "*.inc"))


def _compile_program(name, src, flags):
    exe = os.path.join(TESTS_BUILD, name)
    cmd = [nvcc(), *ARCH, "-O2", "-std=c++17", "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", TESTS_CPP, *flags,
           src, "-o", exe, "-L", BUILD, "-lnebo_gb300", "-Xlinker", "-rpath," + BUILD]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {name}:\n{r.stderr[-4000:]}")
    return exe


def build_programs(verbose=False):
    """Compile the drop-in C++ test programs (needs the library already linked)."""
    os.makedirs(TESTS_BUILD, exist_ok=True)
    deps = _dropin_headers() + glob.glob(os.path.join(INCLUDE, "*.h")) + [LIB]
    jobs = []
    with cf.ThreadPoolExecutor(max_workers=max(1, len(PROGRAMS))) as ex:
        for name, (src, flags) in PROGRAMS.items():
            srcp = os.path.join(TESTS_CPP, src)
            if _stale(os.path.join(TESTS_BUILD, name), [srcp, *deps, __file__]):
                jobs.append(ex.submit(_compile_program, name, srcp, flags))
        for j in jobs:
            j.result()
    if verbose:
        print("built test programs in", TESTS_BUILD)


def build_library(verbose=False, extra_flags=()):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdrs = _headers()
    jobs = []
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        for s in srcs:
            o = os.path.join(BUILD, os.path.basename(s)[:-3] + ".o")
            if _stale(o, [s, *hdrs, __file__]):
                jobs.append(ex.submit(_compile, s, o, extra_flags, True))
        for j in jobs:
            j.result()
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + ".o") for s in srcs]
    if _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build_library(verbose=True)
    if "--programs" in sys.argv:
        build_programs(verbose=True)
    sys.exit(0)
