"""Stencil composition of the `<<=` lowering (Compose in include/spatialops/NeboTiled.h), built for
the host by nvcc from the same header: Interp(Grad(Interp(a))) becomes the 4-point stencil
(g/4) * (-a[i-2] - a[i-1] + a[i] + a[i+1]) of the field; a stencil in x of a stencil in y becomes
the 4 products on the x-y plane; a 125-point composition stays nested.  The coefficients are
checked exactly (every product and sum here is exact in FP64)."""
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
    exe = str(tmp_path_factory.mktemp("compose") / "compose_host")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                    "-I", os.path.join(REPO, "include"), os.path.join(HERE, "cpp", "compose_host.cu"), "-o", exe],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = {}
    for ln in r.stdout.splitlines():
        f = ln.split()
        lines[f[0] if f[0] != "nested" else "nested " + f[1]] = f[1:]
    return lines


def _points(f):
    n = int(f[0])
    pts = {}
    for i in range(n):
        x, y, z, c = f[1 + 4 * i:5 + 4 * i]
        pts[(int(x), int(y), int(z))] = float(c)
    assert len(pts) == n
    return pts


def test_compositions(out):
    g = 1.0 / 3.0
    chain = _points(out["chain"])
    assert set(chain) == {(-2, 0, 0), (-1, 0, 0), (0, 0, 0), (1, 0, 0)}
    for p, c in {(-2, 0, 0): -g / 4, (-1, 0, 0): -g / 4, (0, 0, 0): g / 4, (1, 0, 0): g / 4}.items():
        assert abs(chain[p] - c) <= 1e-16, (p, chain[p], c)
    xy = _points(out["xy"])
    want = {(0, -1, 0): -0.5, (1, -1, 0): 0.5, (0, 0, 0): -1.5, (1, 0, 0): 1.5}
    assert xy == want
    assert "nested box_of_box" in out
