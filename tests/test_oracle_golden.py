"""The oracle (CPU restatement) against golden vectors made by the reference's own Nebo.

Every comparison is bit-exact: same written-cell set (outputs were pre-filled with a sentinel),
same doubles, same reduction values, same error behaviour.
"""
import os

import numpy as np
import pytest

import catalog
import nebo_io
import oracle_dsl as O
from spatialops_gb300 import workloads as W

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _same_bits(a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return a.shape == b.shape and bool((a.view(np.uint64) == b.view(np.uint64)).all())


def _strip_location(msg):
    # the reference appends "\n\t - <file> : <line>" to its messages
    return msg.split("\n\t - ")[0]


@pytest.mark.parametrize("domain", [0, 1, 2])
def test_catalog_matches_reference(domain):
    gold = nebo_io.npz_to_records(np.load(os.path.join(GOLD, f"catalog_d{domain}.npz")))
    mine = catalog.run_catalog(domain)
    assert set(gold) == set(mine)
    for name, g in gold.items():
        m = mine[name]
        assert g[0] == m[0], name
        if g[0] == "field":
            assert g[1] == m[1], name
            assert _same_bits(g[2], m[2]), name
        elif g[0] == "value":
            assert _same_bits(np.float64(g[1]), np.float64(m[1])), name
        else:
            assert _strip_location(g[1]) == _strip_location(m[1]), name


def test_heat_matches_reference():
    z = np.load(os.path.join(GOLD, "heat.npz"))
    T = O.heat_run(z["lam"], z["T0"], tuple(z["n"]), int(z["steps"]), float(z["dt"]))
    assert _same_bits(T, z["f:T"])
    for op in ("sum", "max", "norm"):
        assert O.reduce_field(T, 1, op) == float(z["v:" + op])


def test_heat_threaded_equals_serial():
    z = np.load(os.path.join(GOLD, "heat.npz"))
    T1 = O.heat_run(z["lam"], z["T0"], tuple(z["n"]), int(z["steps"]), float(z["dt"]), threads=1)
    T4 = O.heat_run(z["lam"], z["T0"], tuple(z["n"]), int(z["steps"]), float(z["dt"]), threads=4)
    assert _same_bits(T1, T4)


def test_deep_matches_reference():
    z = np.load(os.path.join(GOLD, "deep.npz"))
    n = tuple(z["n"])
    bits = W.mask_bits_from_points(z["pts"], n)
    out, filt = O.deep_run(z["a"], z["b"], z["c"], bits, n)
    assert _same_bits(out, z["f:out"])
    assert _same_bits(filt, z["f:filt"])
    for op in ("sum", "max", "norm"):
        assert O.reduce_field(filt, 1, op) == float(z["v:" + op])


def test_transport_matches_reference():
    z = np.load(os.path.join(GOLD, "transport.npz"))
    phi = O.transport_run(z["phi0"], z["u"], z["v"], z["w"], z["lam"], int(z["n"]), int(z["steps"]),
                          float(z["dt"]), float(z["nu"]))
    assert _same_bits(phi, z["f:phi"])


def test_mask_bits_layout_matches_bitfield():
    # numpy packing used by the host side == the oracle's BitField restatement
    n = (7, 6, 5)
    pts = nebo_io.mask_points(0, 0, n, 1)
    words = W.mask_bits_from_points(pts, n)
    m = O.Mask.from_points("SVol", pts, (9, 8, 7), 1)
    assert (m.bits[: len(words)] == words).all()


def test_write_limits_deep_chain_negative_ghost():
    # Interp(Grad(Interp(a))) on XVol with one ghost cannot reach the first interior x plane
    n = (8, 8, 8)
    a = O.Field("SVol", np.zeros((10, 10, 10)), 1)
    out = O.Field("XVol", np.zeros((10, 10, 10)), 1)
    db = O.OpDB(n, n)
    i, g = db.interp("SVol", "XVol"), db.grad("XVol", "SVol")
    lim, any_ = O.write_limits(out, i(g(i(a))))
    assert any_ and lim == (1, 8, -1, 9, -1, 9)


# ----------------------------------------------------------------------------- particles
_PARTICLES = np.load(os.path.join(GOLD, "particles.npz"))


def particle_case(name):
    """One case of particles.npz: the inputs of workloads.particle_inputs plus the reference's
    outputs c2p (CellToParticle) and p2c (ParticleToCell, allocation pre-filled with -7777.25)."""
    pre = name + "__"
    return {k[len(pre):]: _PARTICLES[k] for k in _PARTICLES.files if k.startswith(pre)}


PARTICLE_NAMES = [str(c) for c in _PARTICLES["cases"]]


@pytest.mark.parametrize("name", PARTICLE_NAMES)
def test_particles_match_reference(name):
    c = particle_case(name)
    c2p, p2c = O.particle_ops(c)
    assert _same_bits(c2p, c["c2p"]), name
    assert _same_bits(p2c, c["p2c"]), name


def test_particles_reference_known_answers():
    # the reference's own checks (spatialops/particles/test/TestParticleOperators.cpp:86-97)
    c = particle_case("reftest")
    c2p, p2c = O.particle_ops(c)
    assert c2p[0] == 32.5
    assert list(p2c.ravel()[3:13]) == [1, 4, 4, 4, 4, 3, 0, 0, 0, 0]


def test_particles_low_clip_keeps_inside_fraction():
    # a box sticking out of the window's low end by more than one cell: the reference leaves
    # this undefined; the oracle (and the GPU) clip it, so a constant field interpolates to the
    # fraction of the particle inside the window and the scatter deposits that fraction
    c = W.particle_inputs((6, 5, 4), 1, 3, axes=7, seed=3)
    c["cell"][:] = 1.0
    face = c["low"] - c["spacing"] * c["ngm"] - c["spacing"] / 2
    c["psize"][:] = 3.0
    c["px"][:] = face[0] + 0.25   # 1.25 cells out on the low x side
    c["py"][:] = face[1] + 2.5
    c["pz"][:] = face[2] + 2.0
    c2p, p2c = O.particle_ops(c)
    assert np.allclose(c2p, 1.75 / 3.0, rtol=0, atol=1e-15)
    assert abs(p2c.sum() - c["pval"].sum() * 1.75 / 3.0) < 1e-13
