"""The integer-pipe exp and sin of the deep chain, compiled for the host (same source, same
fixed-point arithmetic) and compared with long double expl / sinl: the algorithm's error bound
is checked on the CPU, the GPU build against CUDA's functions in test_gpu_fastmath.py."""
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


@pytest.fixture(scope="module")
def results(tmp_path_factory):
    inc = _cuda_include()
    if shutil.which("g++") is None or inc is None or np.finfo(np.longdouble).nmant < 63:
        pytest.skip("needs g++, the CUDA headers and a long double with a 64-bit significand or more")
    exe = str(tmp_path_factory.mktemp("fixmath") / "fixmath_host")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", inc, "-I", os.path.join(os.path.dirname(HERE), "include"),
                    os.path.join(HERE, "cpp", "fixmath_host.cpp"), "-o", exe],
                   check=True)
    out = subprocess.run([exe, "100000"], check=True, capture_output=True, text=True).stdout
    return {ln.split()[0]: float(ln.split()[1]) for ln in out.splitlines() if ln.strip()}


@pytest.mark.parametrize("name", ["conv_d2f_mismatch", "conv_f2d_mismatch", "table_mismatch"])
def test_bit_built_conversions_match_casts(results, name):
    assert results[name] == 0, (name, results[name])


@pytest.mark.parametrize("name", ["exp_unit", "exp_full", "exp_tiny", "sin_unit", "sin_100", "sin_1e5", "sin_tiny",
                                  "sin_2p20", "sin_near_jpi"])
def test_error_bound(results, name):
    bound = 0.52 if name.startswith("exp") else 1.15
    assert results[name] <= bound, (name, results[name])

