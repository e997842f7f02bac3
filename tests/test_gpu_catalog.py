"""The expression catalog through the drop-in C++ headers on the GPU, against the reference.

tests/cpp/catalog_gpu.cu includes the same tests/cpp/catalog_cases.inc that the reference's own
headers compiled into the golden vectors (tests/golden/catalog_d*.npz), so every case is the
same C++ expression evaluated by the reference's serial Nebo and by one fused sm_103a kernel.

* written-cell sets (outputs were pre-filled with a sentinel) are identical, always;
* error records (the reference's ghost-check exceptions) are identical;
* with NEBO_EXACT_ARITHMETIC (no contraction), arithmetic and stencil results are bit-identical;
  libm functions (sin, exp, pow, ...) differ from the host's by a few ulp;
* in the default build (FMA contraction allowed; the 27-point box sums of the tiled lowering
  split into line sums) every field is within 1e-13 relative max-norm, and max/min values of
  such fields within that field's tolerance.
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

import nebo_io

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(REPO, "tests", "golden")
BUILD = os.path.join(REPO, "tests", "cpp", "_build")

LIBM = {"s_sin", "s_cos", "s_tan", "s_exp", "s_tanh", "s_log", "s_log10", "s_pow", "s_powint"}
CHAINED_LIBM = {"chain_deep_out", "chain_deep_filt"}
EPS = np.finfo(np.float64).eps


@pytest.fixture(scope="module")
def programs():
    import sys

    sys.path.insert(0, os.path.join(REPO, "spatialops-threadfix_gb300"))
    import build as B

    B.build_library()
    B.build_programs()
    return {k: os.path.join(BUILD, k) for k in ("catalog_gpu_exact", "catalog_gpu_fast")}


def _run(exe, domain):
    with tempfile.TemporaryDirectory() as d:
        out = os.path.join(d, "cat.bin")
        subprocess.run([exe, str(domain), out], check=True, timeout=300)
        return nebo_io.read_records(out)


def _strip(msg):
    return msg.split("\n\t - ")[0]


def _check(gold, got, exact):
    assert set(gold) == set(got)
    for name, g in gold.items():
        m = got[name]
        assert g[0] == m[0], name
        if g[0] == "error":
            assert _strip(g[1]) == _strip(m[1]), name
            continue
        if g[0] == "value":
            ref, val = g[1], m[1]
            if "max" in name or "min" in name:
                # exact: the same doubles; default build: the max/min of a field that may differ
                # from the reference's by reassociation (the split box sum, FMA contraction)
                tol = 4 * EPS * abs(ref) if (name == "red_expr_max" or not exact) else 0.0
                if not exact and name.startswith("chain_deep"):
                    tol = 1e-13 * float(np.abs(gold["chain_deep_filt"][2]).max())
            elif name.startswith("chain_deep"):
                tol = 1e-13 * float(np.abs(gold["chain_deep_filt"][2]).sum())
            else:
                tol = 1e-12 * max(1.0, abs(ref))
            assert abs(val - ref) <= tol, (name, val, ref)
            continue
        ga, ma = g[2], m[2]
        assert g[1] == m[1] and ga.shape == ma.shape, name
        sent_g, sent_m = ga == nebo_io.SENTINEL, ma == nebo_io.SENTINEL
        assert (sent_g == sent_m).all(), f"{name}: written-cell set differs"
        w = ~sent_g
        if name in LIBM:
            # a few ulp of each value, or of the field's magnitude where the value is near zero
            scale = float(np.abs(ga[w]).max())
            assert (np.abs(ma[w] - ga[w]) <= 4 * EPS * (np.abs(ga[w]) + scale)).all(), name
        elif exact and name not in CHAINED_LIBM:
            assert (ma[w].view(np.uint64) == ga[w].view(np.uint64)).all(), f"{name}: not bit-identical"
        else:
            scale = max(float(np.abs(ga[w]).max()), 1e-300)
            assert float(np.abs(ma[w] - ga[w]).max()) <= 1e-13 * scale, name


@pytest.mark.parametrize("domain", [0, 1, 2])
def test_catalog_exact_arithmetic(programs, domain):
    gold = nebo_io.npz_to_records(np.load(os.path.join(GOLD, f"catalog_d{domain}.npz")))
    _check(gold, _run(programs["catalog_gpu_exact"], domain), exact=True)


@pytest.mark.parametrize("domain", [0, 1, 2])
def test_catalog_default_build(programs, domain):
    gold = nebo_io.npz_to_records(np.load(os.path.join(GOLD, f"catalog_d{domain}.npz")))
    _check(gold, _run(programs["catalog_gpu_fast"], domain), exact=False)
