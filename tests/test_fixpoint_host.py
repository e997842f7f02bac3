"""The box filter's 128-bit fixed-point helpers (to_units, units_to_double, units_to_double0 in
csrc/fp64_int.cuh), built for the host by nvcc from the same source, against exact rational
arithmetic: to_units rounds x * 2^(1144 - E) to the nearest integer (halves away from zero), and
units_to_double is the correctly rounded (ties to even) double of t * 2^u."""
import os
import shutil
import struct
import subprocess
from fractions import Fraction

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    return None


def _i128(hi, lo):
    v = (int(hi, 16) << 64) | int(lo, 16)
    return v - (1 << 128) if v >> 127 else v


@pytest.fixture(scope="module")
def lines(tmp_path_factory):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("needs nvcc")
    exe = str(tmp_path_factory.mktemp("fixpoint") / "fixpoint_host")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                    "-I", os.path.join(REPO, "include"), "-I", os.path.join(REPO, "spatialops-threadfix_gb300", "csrc"),
                    os.path.join(HERE, "cpp", "fixpoint_host.cu"), "-o", exe], check=True)
    out = subprocess.run([exe, "20000", "11"], check=True, capture_output=True, text=True).stdout
    return [ln.split() for ln in out.splitlines()]


def test_to_units_rounds_exactly(lines):
    n = 0
    for f in lines:
        if f[0] != "U":
            continue
        x = struct.unpack("<d", int(f[1], 16).to_bytes(8, "little"))[0]
        E = int(f[2])
        v = abs(Fraction(x)) * Fraction(2) ** (1144 - E)
        want = int(v + Fraction(1, 2))  # floor(|v| + 1/2): halves away from zero
        want = -want if (int(f[1], 16) >> 63) else want
        assert _i128(f[3], f[4]) == want, f
        n += 1
    assert n == 20000


def test_units_to_double_is_correctly_rounded(lines):
    n = 0
    for f in lines:
        if f[0] != "D":
            continue
        t, u = _i128(f[1], f[2]), int(f[3])
        want = float(Fraction(t) * Fraction(2) ** u)  # Python rounds a Fraction to nearest, ties to even
        got = struct.unpack("<d", int(f[4], 16).to_bytes(8, "little"))[0]
        assert got == want and (got < 0) == (t < 0), (f, want)
        n += 1
    assert n == 20000


def test_zero_sum_is_positive_zero(lines):
    z = [f for f in lines if f[0] == "Z"]
    assert z and int(z[0][1], 16) == 0
