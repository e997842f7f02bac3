"""Generate the golden vectors in this folder from the reference's own Nebo.

Run on the build host, where the reference tree exists:
    python tests/golden/make_golden.py [--ref /root/reference]
It builds oracle/_ref/ref_driver (oracle/Makefile, target `ref`) from the reference's headers,
runs it on small seeded inputs and stores inputs and outputs as compressed .npz fixtures:

  catalog_d{0,1,2}.npz  every case of tests/cpp/catalog_cases.inc on three small domains
                        (7x6x5 / 1 ghost; 6x5x4 / 1 ghost / BC cells on every + face;
                        6^3 / 2 ghosts).  Outputs were pre-filled with -7777.25, so the
                        written-cell set is part of the fixture.
  heat.npz              heat workload at 12x10x8, 20 Euler steps
  deep.npz              deep fused chain at 10x9x8
  transport.npz         scalar transport at 10^3, 2 ghosts, 4 RK2 steps

The GPU machine has no reference tree; it only reads these files.
"""
from __future__ import annotations

import argparse
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "tests"))
sys.path.insert(0, os.path.join(REPO, "spatialops-threadfix_gb300"))

import nebo_io  # noqa: E402
import workloads  # noqa: E402

HEAT_N = (12, 10, 8)
HEAT_STEPS = 20
DEEP_N = (10, 9, 8)
TRANSPORT_N = 10
TRANSPORT_STEPS = 4


def run(cmd):
    subprocess.run(cmd, check=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    run(["make", "-C", os.path.join(REPO, "oracle"), "ref", f"REF={args.ref}"])
    drv = os.path.join(REPO, "oracle", "_ref", "ref_driver")
    with tempfile.TemporaryDirectory() as tmp:
        for d in range(3):
            out = os.path.join(tmp, f"cat{d}.bin")
            run([drv, "catalog", str(d), out])
            np.savez_compressed(os.path.join(HERE, f"catalog_d{d}.npz"),
                                **nebo_io.records_to_npz_dict(nebo_io.read_records(out)))

        lam, T0, dt = workloads.heat_inputs(HEAT_N, sigma=3.0)
        lam.tofile(os.path.join(tmp, "lam.bin"))
        T0.tofile(os.path.join(tmp, "T0.bin"))
        out = os.path.join(tmp, "heat.bin")
        run([drv, "heat", *map(str, HEAT_N), str(HEAT_STEPS), repr(dt),
             os.path.join(tmp, "lam.bin"), os.path.join(tmp, "T0.bin"), out])
        recs = nebo_io.read_records(out)
        np.savez_compressed(os.path.join(HERE, "heat.npz"), n=np.array(HEAT_N), steps=HEAT_STEPS,
                            dt=dt, lam=lam, T0=T0, **nebo_io.records_to_npz_dict(recs))

        a, b, c, pts = workloads.deep_inputs(DEEP_N)
        for name, arr in (("a", a), ("b", b), ("c", c)):
            arr.tofile(os.path.join(tmp, name + ".bin"))
        pts.astype("<i4").tofile(os.path.join(tmp, "pts.bin"))
        out = os.path.join(tmp, "deep.bin")
        run([drv, "deep", *map(str, DEEP_N), *(os.path.join(tmp, s + ".bin") for s in ("a", "b", "c", "pts")), out])
        recs = nebo_io.read_records(out)
        np.savez_compressed(os.path.join(HERE, "deep.npz"), n=np.array(DEEP_N), a=a, b=b, c=c, pts=pts,
                            **nebo_io.records_to_npz_dict(recs))

        phi, u, v, w, lam, dt, nu = workloads.transport_inputs(TRANSPORT_N)
        for name, arr in (("phi", phi), ("u", u), ("v", v), ("w", w), ("lam", lam)):
            arr.tofile(os.path.join(tmp, name + ".bin"))
        out = os.path.join(tmp, "transport.bin")
        run([drv, "transport", str(TRANSPORT_N), str(TRANSPORT_STEPS), repr(dt), repr(nu),
             *(os.path.join(tmp, s + ".bin") for s in ("phi", "u", "v", "w", "lam")), out])
        recs = nebo_io.read_records(out)
        np.savez_compressed(os.path.join(HERE, "transport.npz"), n=TRANSPORT_N, steps=TRANSPORT_STEPS,
                            dt=dt, nu=nu, phi0=phi, u=u, v=v, w=w, lam=lam,
                            **nebo_io.records_to_npz_dict(recs))
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
