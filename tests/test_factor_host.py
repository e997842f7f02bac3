"""Constant-factor pass of the `<<=` lowering (Factor / FactorRoot in include/spatialops/NeboFactor.h),
built for the host by nvcc from the same header.  The face flux Interp(lambda) * Grad(T) becomes
two signed pairs with the factor g/2; the heat update T + dt * Div(flux) one FMA whose ratio is
dt * g * g / 2; unequal pair magnitudes and a zero scalar factor are refused (the launch then
runs the expression as written); a 4-point stencil takes its argument's factor into its weights."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    return None


@pytest.fixture(scope="module")
def out(tmp_path_factory):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("needs nvcc")
    exe = str(tmp_path_factory.mktemp("factor") / "factor_host")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                    "-I", os.path.join(REPO, "include"), os.path.join(HERE, "cpp", "factor_host.cu"), "-o", exe],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    return {ln.split()[0]: ln.split()[1:] for ln in r.stdout.splitlines()}


def test_factoring(out):
    g, dt = 1.0 / 3.0, 0.125
    ok, s, *signs = out["flux"]
    assert ok == "1" and float(s) == 0.5 * g
    assert [float(v) for v in signs] == [1.0, 1.0, -1.0, 1.0]
    ok, r = out["heat"]
    assert ok == "1" and abs(float(r) - dt * g * (0.5 * g)) <= 1e-16
    assert out["unequal"] == ["0"]
    assert out["zero"] == ["0"]
    ok, s, c0, c1 = out["fd4"]
    assert ok == "1" and float(s) == 1.0
    assert float(c0) == 0.5 / 24 and float(c1) == -27.0 * 0.5 / 24
