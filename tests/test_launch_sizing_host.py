"""The z-chunk chooser of the chunked stencil kernels (wave_zchunk, csrc/common.cuh) compiled
for the host: every chosen chunk covers the planes, respects the alignment and the minimum, and
gives six or more waves of resident blocks whenever an admissible chunk does."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME", ""), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


def test_wave_zchunk_sweep(tmp_path):
    inc = _cuda_include()
    if shutil.which("g++") is None or inc is None:
        pytest.skip("needs g++ and the CUDA headers")
    exe = str(tmp_path / "wave_zchunk_host")
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", inc, "-I", os.path.join(REPO, "include"),
                    "-I", os.path.join(REPO, "spatialops-threadfix_gb300", "csrc"),
                    os.path.join(HERE, "cpp", "wave_zchunk_host.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    res = {ln.split()[0]: int(ln.split()[-1]) for ln in out.splitlines() if ln.startswith(("cases", "bad"))}
    assert res["cases"] > 10000
    assert res["bad"] == 0, out
