"""`<<=` on FP32 fields through the drop-in headers (tests/cpp/float_assign.cu), against the same
expressions on FP64 fields with the FP32 inputs rounded from the FP64 ones: the heat update (the
constant factoring on float: signed pairs, FMA sums), a pair with unequal coefficients (the
factoring's fallback), a nested chain (the stencil composition) and a factored operand minus an
unfactored one (r * x - y in one FMA).  The written-cell sets must
be identical and the values within 1e-5 relative max-norm (FP32 rounding); the FP64 results must
equal direct host loops of the expressions to 1e-13."""
import json
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

EXE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cpp", "_build", "float_assign")


@pytest.mark.parametrize("n", [20, 37])
def test_float_assign_matches_double(n):
    assert os.path.exists(EXE), "build the programs first (spatialops-threadfix_gb300/build.py --programs)"
    r = subprocess.run([EXE, str(n)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    d = json.loads(r.stdout.strip().splitlines()[-1])
    for name in ("heat_update", "unequal_pair", "composed_chain", "left_factor_difference"):
        e = d[name]
        print(n, name, e)
        assert e["written"] > 0 and e["write_set_mismatch"] == 0, (name, e)
        assert e["rel_diff"] <= 1e-5, (name, e)
        assert e["fp64_rel_diff_host"] <= 1e-13, (name, e)
