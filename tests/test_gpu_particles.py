"""Particle <-> cell operators on the GPU (nebo_cell_to_particle / nebo_particle_to_cell and the
drop-in ParticleOperators.h) against the reference and the oracle.

* golden cases (tests/golden/particles.npz, made by the reference's own ParticleOperators.h):
  bit-identical through the C ABI and through the drop-in headers (tests/cpp/particles_gpu.cu
  runs the same scene code the reference-built generator ran);
* the reference's own test scene (TestParticleOperators.cpp) with its known answers;
* larger seeded cases, sub-windows, clipped boxes and dense cells: bit-identical to the oracle;
* full size (128^3 cells, 2 M particles): conservation and partition-of-unity properties.
"""
import os
import subprocess
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = np.load(os.path.join(REPO, "tests", "golden", "particles.npz"))
BUILD = os.path.join(REPO, "tests", "cpp", "_build")
NAMES = [str(c) for c in GOLD["cases"]]
FILL = -7777.25


def _case(name):
    pre = name + "__"
    return {k[len(pre):]: GOLD[k] for k in GOLD.files if k.startswith(pre)}


def _same_bits(a, b):
    """Identical doubles; NaN (a zero-size particle divides 0 by 0) matches NaN whatever its
    payload, which differs between the host's and the GPU's division."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    if a.shape != b.shape:
        return False
    na, nb = np.isnan(a), np.isnan(b)
    return bool((na == nb).all() and (a[~na].view(np.uint64) == b[~nb].view(np.uint64)).all())


def _gpu(c, loc="SVol", n=None, ghost=None, bcx=0):
    """Device tensors of one case: (cell Field, px, py, pz, psize, pval)."""
    import torch

    from spatialops_gb300 import Field

    axes = int(c["axes"])
    n = tuple(int(v) for v in (c["n"] if n is None else n))
    ghost = int(c["ghost"] if ghost is None else ghost)
    t = torch.from_numpy(np.ascontiguousarray(c["cell"], dtype=np.float64)).cuda()
    cell = Field(loc, n, ghost, (int(bcx), 0, 0), tensor=t)
    dev = [torch.from_numpy(np.ascontiguousarray(c[k], dtype=np.float64)).cuda() for k in ("px", "py", "pz")]
    pos = [dev[a] if (axes >> a) & 1 else None for a in range(3)]
    psize = torch.from_numpy(np.ascontiguousarray(c["psize"], dtype=np.float64)).cuda()
    pval = torch.from_numpy(np.ascontiguousarray(c["pval"], dtype=np.float64)).cuda()
    return cell, pos[0], pos[1], pos[2], psize, pval


def _run_both(c, **kw):
    """(c2p, p2c) on the GPU; p2c's allocation pre-filled with FILL."""
    import torch

    import spatialops_gb300 as S
    from spatialops_gb300 import Field

    cell, px, py, pz, psize, pval = _gpu(c, **kw)
    dest = torch.full((psize.numel(),), FILL, dtype=torch.float64, device="cuda")
    S.cell_to_particle(cell, px, py, pz, psize, dest, c["spacing"], c["low"])
    out = Field(cell.loc, cell.n, cell.ghost, cell.bc, tensor=torch.full_like(cell.tensor, FILL))
    S.particle_to_cell(pval, px, py, pz, psize, out, c["spacing"], c["low"])
    torch.cuda.synchronize()
    return dest.cpu().numpy(), out.numpy()


@pytest.mark.parametrize("name", NAMES)
def test_golden_cases_bit_exact_c_abi(name):
    c = _case(name)
    loc = "SVol" if str(c["field"]) == "svol" else "XVol"
    c2p, p2c = _run_both(c, loc=loc, bcx=int(c["bcx"]))
    assert _same_bits(c2p, c["c2p"]), name
    assert _same_bits(p2c, c["p2c"]), name


@pytest.fixture(scope="module")
def program():
    import sys

    sys.path.insert(0, os.path.join(REPO, "spatialops-threadfix_gb300"))
    import build as B

    B.build_library()
    B.build_programs()
    return os.path.join(BUILD, "particles_gpu")


@pytest.mark.parametrize("name", NAMES)
def test_golden_cases_bit_exact_dropin(program, name):
    c = _case(name)
    npart = len(c["psize"])
    with tempfile.TemporaryDirectory() as d:
        files = []
        for key in ("cell", "px", "py", "pz", "psize", "pval"):
            path = os.path.join(d, key + ".bin")
            np.ascontiguousarray(c[key], dtype="<f8").tofile(path)
            files.append(path)
        out = os.path.join(d, "out.bin")
        ctor = [repr(float(v)) for v in c["ctor"]]  # the operators' constructor arguments
        subprocess.run([program, "scene", "0" if str(c["field"]) == "svol" else "1", *map(str, c["n"]),
                        str(int(c["ghost"])), str(int(c["bcx"])), str(npart), str(int(c["axes"])), *ctor, *files,
                        out],
                       check=True, timeout=300)
        r = np.fromfile(out, dtype="<f8")
    assert _same_bits(r[:npart], c["c2p"]), name
    assert _same_bits(r[npart:].reshape(c["p2c"].shape), c["p2c"]), name


def test_reference_test_scene(program):
    # spatialops/particles/test/TestParticleOperators.cpp:22-99 on the drop-in headers
    r = subprocess.run([program, "reftest"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "PASS" in r.stdout, r.stdout + r.stderr


@pytest.mark.parametrize("spill,seed", [(False, 21), (True, 22)])
def test_random_cases_match_oracle(spill, seed):
    import oracle_dsl as O
    from spatialops_gb300 import workloads as W

    n, g = (40, 36, 30), 2
    c = W.particle_inputs(n, g, 60000, axes=7, spacing=(0.21, 0.33, 0.27), low=(-1.0, 2.0, 0.5),
                          size_range=(0.3, 3.0), seed=seed, spill=spill)
    c["n"], c["ghost"] = np.array(n), g
    want_c2p, want_p2c = O.particle_ops(c)
    c2p, p2c = _run_both(c)
    assert _same_bits(c2p, want_c2p)
    assert _same_bits(p2c, want_p2c)


def test_low_clip_and_far_particles_match_oracle():
    # boxes more than a cell below the window (undefined in the reference; clipped here and in
    # the oracle), boxes wholly outside on either side, and zero-size particles
    import oracle_dsl as O
    from spatialops_gb300 import workloads as W

    n, g = (10, 9, 8), 1
    c = W.particle_inputs(n, g, 400, axes=7, seed=5)
    c["n"], c["ghost"] = np.array(n), g
    rng = np.random.default_rng(6)
    face = c["low"] - c["spacing"] * c["ngm"] - c["spacing"] / 2
    for a, k in enumerate(("px", "py", "pz")):
        sel = rng.random(400) < 0.3
        c[k][sel] = face[a] + rng.uniform(-4.0, 14.0, sel.sum())
    c["psize"][:20] = 0.0
    want_c2p, want_p2c = O.particle_ops(c)
    c2p, p2c = _run_both(c)
    assert _same_bits(c2p, want_c2p)
    assert _same_bits(p2c, want_p2c)


def test_subwindow_matches_oracle():
    # a cell field whose window is a sub-box of its allocation: only window cells are written
    import torch

    import oracle_dsl as O
    import spatialops_gb300 as S
    from spatialops_gb300 import NeboField, workloads as W

    glob, off, ext = (20, 18, 16), (2, 1, 3), (14, 12, 10)
    c = W.particle_inputs((ext[0] - 2, ext[1] - 2, ext[2] - 2), 1, 3000, axes=7, seed=8, spill=True)
    rng = np.random.default_rng(9)
    full = rng.uniform(-1, 1, size=glob[::-1])
    full[off[2]:off[2] + ext[2], off[1]:off[1] + ext[1], off[0]:off[0] + ext[0]] = c["cell"]
    c["cell"], c["glob"] = full, np.array(glob)
    want_c2p, want_p2c = O.particle_ops(c, off=off, nmax=ext)

    def desc(t):
        d = NeboField()
        d.data = t.data_ptr()
        d.glob[:], d.offset[:], d.extent[:] = glob, off, ext
        d.ghost_minus[:] = d.ghost_plus[:] = (1, 1, 1)
        d.has_bc[:] = d.bc_extra[:] = (0, 0, 0)
        d.dtype = 0
        return d

    t = torch.from_numpy(full).cuda()
    pos = [torch.from_numpy(c[k]).cuda() for k in ("px", "py", "pz")]
    psize = torch.from_numpy(c["psize"]).cuda()
    pval = torch.from_numpy(c["pval"]).cuda()
    dest = torch.empty(3000, dtype=torch.float64, device="cuda")
    S.cell_to_particle(desc(t), *pos, psize, dest, c["spacing"], c["low"], ghost_minus=c["ngm"])
    o = torch.full_like(t, FILL)
    S.particle_to_cell(pval, *pos, psize, desc(o), c["spacing"], c["low"], ghost_minus=c["ngm"])
    torch.cuda.synchronize()
    assert _same_bits(dest.cpu().numpy(), want_c2p)
    assert _same_bits(o.cpu().numpy(), want_p2c)


def test_no_particles():
    import torch

    import spatialops_gb300 as S
    from spatialops_gb300 import Field

    cell = Field("SVol", (5, 4, 3), 1, tensor=torch.full((5, 6, 7), FILL, dtype=torch.float64, device="cuda"))
    e = torch.empty(0, dtype=torch.float64, device="cuda")
    S.particle_to_cell(e, e, e, e, e, cell, (1, 1, 1), (0.5, 0.5, 0.5))
    S.cell_to_particle(cell, e, e, e, e, e, (1, 1, 1), (0.5, 0.5, 0.5))
    torch.cuda.synchronize()
    a = cell.numpy()
    assert (a == 0).all() and not np.signbit(a).any()  # the reference's dest <<= 0


def test_dense_cells_deterministic():
    # ~200 particles per cell: long per-cell entry lists, repeated runs give the same bits
    import oracle_dsl as O
    from spatialops_gb300 import workloads as W

    n, g = (6, 6, 6), 1
    c = W.particle_inputs(n, g, 40000, axes=7, spacing=(0.5, 0.5, 0.5), low=(0.25, 0.25, 0.25),
                          size_range=(0.5, 3.0), seed=31)
    c["n"], c["ghost"] = np.array(n), g
    want_c2p, want_p2c = O.particle_ops(c)
    for _ in range(3):
        c2p, p2c = _run_both(c)
        assert _same_bits(c2p, want_c2p)
        assert _same_bits(p2c, want_p2c)


def test_full_size_properties():
    # 128^3 cells + 1 ghost, 2 M particles inside the window: ParticleToCell conserves the total
    # (each particle's weights sum to one), CellToParticle of a constant is that constant, and
    # scaling the field by a power of two scales the result exactly
    import torch

    import spatialops_gb300 as S
    from spatialops_gb300 import Field

    n, g, npart = (128, 128, 128), 1, 2_000_000
    gen = torch.Generator(device="cuda").manual_seed(41)
    d = 1.0 / 128
    face = 0.5 * d - d * g - d / 2
    span = (n[0] + 2 * g) * d
    size = torch.rand(npart, generator=gen, device="cuda", dtype=torch.float64) * 2.0 * d + 0.2 * d
    pos = [face + size / 2 + torch.rand(npart, generator=gen, device="cuda", dtype=torch.float64) * (span - size)
           for _ in range(3)]
    pval = torch.rand(npart, generator=gen, device="cuda", dtype=torch.float64) + 0.5
    cell = Field("SVol", n, g)
    S.particle_to_cell(pval, *pos, size, cell, (d, d, d), (0.5 * d,) * 3)
    total = cell.tensor.sum().item()
    assert abs(total - pval.sum().item()) <= 1e-12 * abs(total)
    cell.tensor.fill_(1.0)
    out = torch.empty(npart, dtype=torch.float64, device="cuda")
    S.cell_to_particle(cell, *pos, size, out, (d, d, d), (0.5 * d,) * 3)
    # the weights come from coordinate differences, so they sum to one only to ~1e-13; the
    # reference's debug check allows 1e-10 (ParticleOperators.h:270, 395)
    assert (out - 1.0).abs().max().item() < 1e-10
    cell.tensor.copy_(torch.rand(cell.tensor.shape, generator=gen, device="cuda", dtype=torch.float64))
    S.cell_to_particle(cell, *pos, size, out, (d, d, d), (0.5 * d,) * 3)
    ref = out.clone()
    cell.tensor.mul_(8.0)
    S.cell_to_particle(cell, *pos, size, out, (d, d, d), (0.5 * d,) * 3)
    assert torch.equal(out, ref * 8.0)
