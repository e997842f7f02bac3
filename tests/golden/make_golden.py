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
  particles.npz         CellToParticle / ParticleToCell (oracle/_ref/ref_particles) on the cases
                        of PARTICLE_CASES, incl. the reference's own 1-D test scene

Machines without the reference tree (where the GPU tests run) only read these files.
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

# name -> (field, n, ghost, bcx, nparticles, axes, ctor (dx, xlo, dy, ylo, dz, zlo), size_range, spill, seed)
PARTICLE_CASES = {
    "svol3d": ("svol", (12, 10, 8), 1, False, 300, 7, (0.37, 1.3, 0.5, -2.0, 0.29, 0.7), (0.3, 2.5), False, 11),
    "svol2d": ("svol", (9, 7, 1), 2, False, 200, 3, (0.25, 0.0, 0.4, 1.0, -1.0, 0.0), (0.3, 2.5), False, 12),
    "zoff3d": ("svol", (7, 6, 5), 1, False, 120, 3, (1.0, 0.5, 1.0, 0.5, -1.0, 0.0), (0.4, 1.8), False, 13),
    "spill": ("svol", (8, 7, 6), 1, False, 250, 7, (1.0, 0.5, 1.0, 0.5, 1.0, 0.5), (0.3, 2.0), True, 14),
    "dense": ("svol", (4, 4, 4), 1, False, 600, 7, (0.5, 0.25, 0.5, 0.25, 0.5, 0.25), (0.5, 2.5), False, 15),
    "xvol_bc": ("xvol", (6, 5, 4), 1, True, 150, 7, (1.0, 0.0, 1.0, 0.5, 1.0, 0.5), (0.3, 2.0), True, 16),
    "yonly": ("svol", (1, 12, 1), 1, False, 40, 2, (-1.0, 0.0, 0.75, 0.375, -1.0, 0.0), (0.3, 3.0), True, 17),
}


def particle_state(ctor):
    """Spacing and low coordinate after the operators' constructor (ParticleOperators.h:152-166 and 277-291)."""
    d, lo = [], []
    for a in range(3):
        da, la = ctor[2 * a], ctor[2 * a + 1]
        d.append(1.0 if da <= 0 else da)
        lo.append(0.0 if da <= 0 else la)
    return tuple(d), tuple(lo)


def particle_goldens(drv, tmp):
    out = {}
    # the reference's own scene (spatialops/particles/test/TestParticleOperators.cpp:22-99): 10 cells
    # of width 1, 3 ghosts, cell value 10*x, one particle at x=3.25 of size 5 carrying 20
    cases = dict(PARTICLE_CASES)
    cases["reftest"] = ("svol", (10, 1, 1), 3, False, 1, 1, (1.0, 0.5, -1.0, 0.0, -1.0, 0.0), None, False, 0)
    for name, (field, n, g, bcx, npart, axes, ctor, size_range, spill, seed) in cases.items():
        spacing, low = particle_state(ctor)
        if name == "reftest":
            glob, ngm = workloads.particle_window(n, g)
            x = np.arange(glob[0]) - g + 0.5
            d = dict(glob=np.array(glob), ngm=np.array(ngm), cell=(10 * x).reshape(1, 1, -1),
                     px=np.array([3.25]), py=np.zeros(1), pz=np.zeros(1), psize=np.array([5.0]),
                     pval=np.array([20.0]), axes=axes, spacing=np.array(spacing), low=np.array(low))
        else:
            d = workloads.particle_inputs(n, g, npart, axes=axes, spacing=spacing, low=low, size_range=size_range,
                                          seed=seed, spill=spill, field=field, bcx=bcx)
        files = []
        for key in ("cell", "px", "py", "pz", "psize", "pval"):
            path = os.path.join(tmp, f"p_{name}_{key}.bin")
            np.ascontiguousarray(d[key], dtype="<f8").tofile(path)
            files.append(path)
        res = os.path.join(tmp, f"p_{name}_out.bin")
        run([drv, "scene", "0" if field == "svol" else "1", *map(str, n), str(g), str(int(bcx)), str(npart), str(axes),
             *map(repr, ctor), *files, res])
        r = np.fromfile(res, dtype="<f8")
        for key, v in d.items():
            out[f"{name}__{key}"] = np.asarray(v)
        out[f"{name}__c2p"] = r[:npart]
        out[f"{name}__p2c"] = r[npart:].reshape(d["cell"].shape)
        out[f"{name}__field"] = np.array(field)
        out[f"{name}__n"] = np.array(n)
        out[f"{name}__ghost"] = np.array(g)
        out[f"{name}__bcx"] = np.array(int(bcx))
        out[f"{name}__ctor"] = np.array(ctor, dtype=float)
    np.savez_compressed(os.path.join(HERE, "particles.npz"), cases=np.array(sorted(cases)), **out)


def run(cmd):
    subprocess.run(cmd, check=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("NEBO_REFERENCE", "/root/reference"))
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
        particle_goldens(os.path.join(REPO, "oracle", "_ref", "ref_particles"), tmp)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
