"""The scalar-transport configuration written in Nebo (tests/cpp/transport_dropin.cu: user stencil
builders for the 4th-order gradient and the upwind reads, cond on the face velocity, Heun's RK2
with periodic fills) through the drop-in headers, against the golden vectors the same code
produced through the reference's own Nebo (tests/golden/transport.npz): within 1e-13 relative
max-norm over the whole window."""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
EXE = os.path.join(HERE, "cpp", "_build", "transport_dropin")


def test_transport_written_in_nebo_matches_reference_golden(tmp_path):
    assert os.path.exists(EXE), "build the programs first (spatialops-threadfix_gb300/build.py --programs)"
    z = np.load(os.path.join(HERE, "golden", "transport.npz"))
    n, steps = int(z["n"]), int(z["steps"])
    paths = []
    for name in ("phi0", "u", "v", "w", "lam"):
        p = str(tmp_path / f"{name}.bin")
        np.ascontiguousarray(z[name], dtype="<f8").tofile(p)
        paths.append(p)
    out = str(tmp_path / "phi.bin")
    r = subprocess.run([EXE, "check", str(n), str(steps), repr(float(z["dt"])), repr(float(z["nu"])), *paths, out],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(out, dtype="<f8")
    want = np.ascontiguousarray(z["f:phi"], dtype=np.float64).reshape(-1)
    assert got.shape == want.shape
    err = float(np.abs(got - want).max() / np.abs(want).max())
    print(f"transport through <<= ({n}^3, {steps} RK2 steps): rel max-norm err vs the reference golden {err:.2e}")
    assert err <= 1e-13
