"""bench.py's reference arm on the host (no GPU needed): one JSON line with the contract's keys,
naming the same workload as the device arm."""
import json
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _line(*args):
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", *args], check=True, capture_output=True, text=True, cwd=REPO,
                         timeout=600).stdout
    lines = [ln for ln in out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out
    return json.loads(lines[0])


@pytest.mark.parametrize("workload", ["deep", "particles", "heat32", "transport32", "patches", "adjoint"])
def test_reference_arm_line(workload):
    sys.path.insert(0, REPO)
    import bench

    d = _line("--workload", workload)
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["warmup"] >= 3
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0
    n = bench.N_DEFAULT
    bench.graft._import_pkg()
    from spatialops_gb300 import workloads as W

    cells = int(sum(int(a) * int(b) * int(c) for a, b, c in W.patch_shapes(512)))
    want = {"deep": bench.deep_label(n), "particles": bench.particles_label(n, n ** 3),
            "heat32": bench.heat_label(n, "f32"), "transport32": bench.transport_label(n, "f32"),
            "patches": bench.patches_label(512, cells, "f64"), "adjoint": bench.adjoint_label(192, 500)}[workload]
    assert d["config"]["workload"] == want
    metric = {"particles": "particle cell<->particle exchanges/s",
              "adjoint": "adjoint gradient forward-cell-steps/s"}.get(workload, f"{workload} cell-updates/s")
    assert d["metric"] == metric
