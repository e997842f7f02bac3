"""The heat and scalar-transport configurations written in Nebo (tests/cpp/configs_dropin.cu), the
code that produced tests/golden/heat.npz and transport.npz through the reference's own Nebo, run
through the drop-in headers:
* heat: T' <<= T + dt * (DivX(InterpX(lambda) * GradX(T)) + ...) with the operator database's
  operators and periodic fills, 20 steps, then nebo_sum/max/norm;
* deep: out <<= cond(mask, 0)(Interp(Grad(Interp(a))) * exp(b) + sin(c)), filt <<= BoxFilter(out),
  then nebo_sum/max/norm (exp and sin within their ulp bounds of the host's libm, so 1e-13);
* transport: user stencil builders for the 4th-order gradient and the upwind reads, cond on the
  face velocity, Heun's RK2 with periodic fills.
Fields within 1e-13 relative max-norm of the goldens over the whole window (the default build
reassociates: composed stencils, factored constants); reductions within 1e-13."""
import json
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
EXE = os.path.join(HERE, "cpp", "_build", "configs_dropin")


def _write(tmp_path, z, names):
    paths = []
    for name in names:
        p = str(tmp_path / f"{name}.bin")
        np.ascontiguousarray(z[name], dtype="<f8").tofile(p)
        paths.append(p)
    return paths


def _rel(got, want):
    return float(np.abs(got - want).max() / np.abs(want).max())


def test_heat_written_in_nebo_matches_reference_golden(tmp_path):
    assert os.path.exists(EXE), "build the programs first (spatialops-threadfix_gb300/build.py --programs)"
    z = np.load(os.path.join(HERE, "golden", "heat.npz"))
    n = [int(v) for v in z["n"]]
    out = str(tmp_path / "T.bin")
    r = subprocess.run([EXE, "heat", *map(str, n), str(int(z["steps"])), repr(float(z["dt"])),
                        *_write(tmp_path, z, ("lam", "T0")), out], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    red = json.loads(r.stdout.strip().splitlines()[-1])
    err = _rel(np.fromfile(out, dtype="<f8"), np.ascontiguousarray(z["f:T"]).reshape(-1))
    print(f"heat through <<= ({n}, {int(z['steps'])} steps): rel max-norm err vs the reference golden {err:.2e}; "
          f"reductions {red}")
    assert err <= 1e-13
    mag = float(np.abs(z["f:T"]).sum())
    assert abs(red["sum"] - float(z["v:sum"])) <= 1e-13 * mag
    assert abs(red["max"] - float(z["v:max"])) <= 1e-13 * abs(float(z["v:max"]))
    assert abs(red["norm"] - float(z["v:norm"])) <= 1e-13 * float(z["v:norm"])


def test_deep_written_in_nebo_matches_reference_golden(tmp_path):
    assert os.path.exists(EXE), "build the programs first (spatialops-threadfix_gb300/build.py --programs)"
    z = np.load(os.path.join(HERE, "golden", "deep.npz"))
    n = [int(v) for v in z["n"]]
    pts = str(tmp_path / "pts.bin")
    np.ascontiguousarray(z["pts"], dtype="<i4").tofile(pts)
    out, filt = str(tmp_path / "out.bin"), str(tmp_path / "filt.bin")
    r = subprocess.run([EXE, "deep", *map(str, n), *_write(tmp_path, z, ("a", "b", "c")), pts, out, filt],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    red = json.loads(r.stdout.strip().splitlines()[-1])
    e_out = _rel(np.fromfile(out, dtype="<f8"), np.ascontiguousarray(z["f:out"]).reshape(-1))
    e_filt = _rel(np.fromfile(filt, dtype="<f8"), np.ascontiguousarray(z["f:filt"]).reshape(-1))
    print(f"deep chain through <<= ({n}): rel max-norm err vs the reference golden out {e_out:.2e}, "
          f"filt {e_filt:.2e}; reductions {red}")
    assert e_out <= 1e-13 and e_filt <= 1e-13
    mag = float(np.abs(z["f:filt"]).sum())
    assert abs(red["sum"] - float(z["v:sum"])) <= 1e-13 * mag
    assert abs(red["max"] - float(z["v:max"])) <= 1e-13 * abs(float(z["v:max"]))
    assert abs(red["norm"] - float(z["v:norm"])) <= 1e-13 * float(z["v:norm"])


def test_transport_written_in_nebo_matches_reference_golden(tmp_path):
    assert os.path.exists(EXE), "build the programs first (spatialops-threadfix_gb300/build.py --programs)"
    z = np.load(os.path.join(HERE, "golden", "transport.npz"))
    n, steps = int(z["n"]), int(z["steps"])
    out = str(tmp_path / "phi.bin")
    r = subprocess.run([EXE, "transport", str(n), str(steps), repr(float(z["dt"])), repr(float(z["nu"])),
                        *_write(tmp_path, z, ("phi0", "u", "v", "w", "lam")), out],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    err = _rel(np.fromfile(out, dtype="<f8"), np.ascontiguousarray(z["f:phi"]).reshape(-1))
    print(f"transport through <<= ({n}^3, {steps} RK2 steps): rel max-norm err vs the reference golden {err:.2e}")
    assert err <= 1e-13
