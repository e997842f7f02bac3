"""Deep fused chain (cond + mask + Interp(Grad(Interp)) * exp + sin, box filter) on the GPU."""
import os

import numpy as np
import pytest

import oracle_dsl as O
import spatialops_gb300 as N
from spatialops_gb300 import workloads as W

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-13  # relative max-norm (FMA/reassociation and CUDA's exp/sin vs the host libm)


def _relerr(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _gpu(a, b, c, pts, n, dx=1.0):
    A = N.Field.from_numpy("SVol", a, 1)
    B = N.Field.from_numpy("XVol", b, 1)
    C = N.Field.from_numpy("XVol", c, 1)
    out = N.Field("XVol", n, 1)
    filt = N.Field("XVol", n, 1)
    words = N.mask_from_points(N.mask_words(out.glob), out.glob, 1, pts)
    N.deep_chain(A, B, C, words, out, filt, dx)
    return out, filt, words


def test_deep_vs_reference_golden():
    z = np.load(os.path.join(GOLD, "deep.npz"))
    n = tuple(int(v) for v in z["n"])
    out, filt, _ = _gpu(z["a"], z["b"], z["c"], z["pts"], n)
    o, f = out.numpy(), filt.numpy()
    g_out, g_filt = z["f:out"], z["f:filt"]
    # written-cell set: masked cells are exactly zero, and the unwritten x=0 plane stays zero
    assert ((o == 0.0) == (g_out == 0.0)).all()
    assert _relerr(o, g_out) <= TOL
    assert _relerr(f, g_filt) <= TOL
    assert abs(N.nebo_sum(filt) - float(z["v:sum"])) <= TOL * float(np.abs(g_filt).sum())
    assert abs(N.nebo_max(filt) - float(z["v:max"])) <= TOL * abs(float(z["v:max"]))
    assert abs(N.nebo_norm(filt) - float(z["v:norm"])) <= TOL * float(z["v:norm"])


def test_mask_words_match_bitfield_layout():
    n = (37, 12, 9)
    _, _, _, pts = W.deep_inputs(n)
    words = N.mask_from_points(N.mask_words(N.glob_dims("XVol", n, 1)), N.glob_dims("XVol", n, 1), 1, pts)
    ref = W.mask_bits_from_points(pts, n)
    assert (words.cpu().numpy().view(np.uint32) == ref).all()


# thin and ragged shapes: one or two tiles, runs of the filter's flat split crossing tiles, a
# chain z split larger than a block's plane count
@pytest.mark.parametrize("n", [(64, 64, 64), (45, 30, 17), (33, 5, 2), (130, 3, 9), (8, 70, 3)])
def test_deep_vs_oracle(n):
    a, b, c, pts = W.deep_inputs(n)
    out, filt, _ = _gpu(a, b, c, pts, n)
    o_out, o_filt = O.deep_run(a, b, c, W.mask_bits_from_points(pts, n), n)
    assert _relerr(out.numpy(), o_out) <= TOL
    assert _relerr(filt.numpy(), o_filt) <= TOL


NAN_SENTINEL = np.uint64(0x7FF4DEAD00C0FFEE)  # a NaN payload no computed value carries


@pytest.mark.parametrize("n", [(64, 64, 64), (45, 30, 17), (33, 5, 2), (130, 3, 9), (8, 70, 3)])
def test_deep_written_cells_with_sentinel(n):
    """out and filt pre-filled with a NaN payload: the cells still holding it are exactly those
    outside the reference's write regions (calculate_actual_ghost through the oracle for out; the
    interior for filt), so an extra or a missing write of any value fails."""
    import torch

    a, b, c, pts = W.deep_inputs(n)
    A = N.Field.from_numpy("SVol", a, 1)
    B = N.Field.from_numpy("XVol", b, 1)
    C = N.Field.from_numpy("XVol", c, 1)
    g = N.glob_dims("XVol", n, 1)

    def sentinel_field():
        t = torch.full((g[2], g[1], g[0]), int(NAN_SENTINEL.astype(np.int64)), dtype=torch.int64, device="cuda")
        return N.Field("XVol", n, 1, tensor=t.view(torch.float64))

    out, filt = sentinel_field(), sentinel_field()
    words = N.mask_from_points(N.mask_words(out.glob), out.glob, 1, pts)
    N.deep_chain(A, B, C, words, out, filt)
    lim = O.deep_write_region(n)
    want = np.ones((g[2], g[1], g[0]), dtype=bool)
    want[lim[4] + 1:lim[5] + 1, lim[2] + 1:lim[3] + 1, lim[0] + 1:lim[1] + 1] = False
    assert np.array_equal(out.numpy().view(np.uint64) == NAN_SENTINEL, want), (n, lim)
    # the filter writes the interior only (cells next to out's unwritten planes read the payload
    # and come out as quiet NaNs, never as the payload itself)
    want_f = np.ones_like(want)
    want_f[1:-1, 1:-1, 1:-1] = False
    assert np.array_equal(filt.numpy().view(np.uint64) == NAN_SENTINEL, want_f), n


@pytest.mark.parametrize("n,interior", [((64, 64, 64), False), ((45, 30, 17), False), ((45, 30, 17), True),
                                        ((33, 5, 2), False), ((130, 3, 9), True), ((8, 70, 3), False)])
def test_fused_filter_reductions(n, interior):
    """nebo_deep_chain_reduce: filt bit-identical to the unfused chain; {sum, max, min, norm} of
    filt (its stale ghost cells included unless interior) equal to the one-pass reductions of
    the written field, and to the oracle's serial folds within the reduction tolerance."""
    import torch

    a, b, c, pts = W.deep_inputs(n)
    out1, filt1, words = _gpu(a, b, c, pts, n)
    A = N.Field.from_numpy("SVol", a, 1)
    B = N.Field.from_numpy("XVol", b, 1)
    C = N.Field.from_numpy("XVol", c, 1)
    out2 = N.Field("XVol", n, 1)
    # ghost cells of filt hold values the filter never writes; the ghost-inclusive reductions see them
    stale = np.random.default_rng(11).uniform(-3.0, 5.0, size=filt1.numpy().shape)
    filt2 = N.Field.from_numpy("XVol", stale, 1)
    red = torch.zeros(4, dtype=torch.float64, device="cuda")
    N.deep_chain(A, B, C, words, out2, filt2, reductions=red, interior=interior)
    f2 = filt2.numpy()
    core = (slice(1, -1),) * 3
    assert (f2[core].view(np.int64) == filt1.numpy()[core].view(np.int64)).all()
    if not interior:
        shell = np.ones(f2.shape, bool)
        shell[core] = False
        assert (f2[shell] == stale[shell]).all()
    got = red.cpu().numpy()
    ref = torch.zeros(4, dtype=torch.float64, device="cuda")
    N.reduce_all(filt2, interior, ref)
    ref = ref.cpu().numpy()
    scale = float(np.abs(f2[core] if interior else f2).sum())
    assert abs(got[0] - ref[0]) <= 1e-13 * scale
    assert got[1] == ref[1] and got[2] == ref[2]
    assert abs(got[3] - ref[3]) <= 1e-13 * ref[3]
    assert got[1] == O.reduce_field(f2, 1, "max", interior)
    assert got[2] == O.reduce_field(f2, 1, "min", interior)
    assert abs(got[0] - O.reduce_field(f2, 1, "sum", interior)) <= 1e-13 * scale
    o_norm = O.reduce_field(f2, 1, "norm", interior)
    assert abs(got[3] - o_norm) <= 1e-13 * o_norm


# ----------------------------------------------------------------------------- standalone filter
FILL = -7777.25


def _filter_inputs(kind, n, seed):
    """An XVol window (1 ghost) of one of several value distributions."""
    rng = np.random.default_rng(seed)
    g = O.glob_dims("XVol", n, 1, (0, 0, 0))
    shp = (g[2], g[1], g[0])
    if kind == "uniform":
        return rng.uniform(-1.0, 1.0, shp)
    if kind == "spikes":  # ambient values near 1 and a few cells 1e18 larger in the same tiles
        a = rng.uniform(0.5, 1.5, shp)
        idx = rng.integers(0, a.size, 40)
        a.flat[idx] = 1e18
        return a
    if kind == "range20":  # |values| spread over 10^-10 .. 10^10, random signs
        return 10.0 ** rng.uniform(-10, 10, shp) * rng.choice([-1.0, 1.0], shp)
    if kind == "special":  # inf, -inf and NaN cells, an all-zero plane, a plane of subnormals
        a = rng.uniform(-1.0, 1.0, shp)
        a.flat[rng.integers(0, a.size, 3)] = np.inf
        a.flat[rng.integers(0, a.size, 3)] = -np.inf
        a.flat[rng.integers(0, a.size, 3)] = np.nan
        a[4] = 0.0
        a[7] = rng.uniform(-1.0, 1.0, a[7].shape) * 2.0 ** -1070
        a[9] = rng.uniform(-1.0, 1.0, a[9].shape) * 2.0 ** -900
        return a
    raise ValueError(kind)


def _oracle_filter(src, n):
    db = O.OpDB(n, n)
    lhs = O.Field("XVol", np.full_like(src, FILL), 1)
    O.assign(lhs, db.filter()(O.Field("XVol", np.ascontiguousarray(src), 1)))
    return lhs.data


def _local_abs(src):
    """sum over the 27 neighbours of |src| / 27 at every interior cell (ghost layer: 0)."""
    a = np.abs(np.nan_to_num(src, nan=0.0, posinf=0.0, neginf=0.0))
    out = np.zeros_like(a)
    inner = (slice(1, -1),) * 3
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                out[inner] += a[1 + dz:a.shape[0] - 1 + dz, 1 + dy:a.shape[1] - 1 + dy, 1 + dx:a.shape[2] - 1 + dx]
    return out / 27.0


@pytest.mark.parametrize("kind", ["uniform", "spikes", "range20", "special"])
def test_box_filter_matches_oracle(kind):
    # the 128-bit fixed-point sums against the oracle's FP64 sums, cell by cell: within 1e-13 of
    # the local magnitude sum (the scale of either side's rounding), same written cells, same
    # infinities and NaNs
    import torch

    n = (45, 37, 21)
    src = _filter_inputs(kind, n, 17)
    want = _oracle_filter(src, n)
    S = N.Field.from_numpy("XVol", src, 1)
    D = N.Field.from_numpy("XVol", np.full_like(src, FILL), 1)
    red = torch.zeros(4, dtype=torch.float64, device="cuda")
    N.box_filter(S, D, reductions=red)
    got = D.numpy()
    assert np.array_equal(np.isnan(got), np.isnan(want))
    fin = np.isfinite(want)
    assert np.array_equal(got[~fin & ~np.isnan(want)], want[~fin & ~np.isnan(want)])  # signed infinities
    tol = 1e-13 * _local_abs(src) + 1e-300
    assert (np.abs(got[fin] - want[fin]) <= tol[fin]).all(), float(np.max(np.abs(got[fin] - want[fin]) / tol[fin]))
    if kind != "special":
        r = red.cpu().numpy()  # dst's ghost cells (FILL) are part of the ghost-inclusive reductions
        assert r[1] == O.reduce_field(got, 1, "max") and r[2] == O.reduce_field(got, 1, "min")
        assert abs(r[0] - O.reduce_field(got, 1, "sum")) <= 1e-13 * np.abs(got).sum()
        assert abs(r[3] - O.reduce_field(got, 1, "norm")) <= 1e-13 * O.reduce_field(got, 1, "norm")


def test_box_filter_is_the_deep_chain_filter():
    # nebo_box_filter on the chain's `out` gives the chain's own `filt` bit for bit
    n = (40, 24, 18)
    a, b, c, pts = W.deep_inputs(n)
    A = N.Field.from_numpy("SVol", a, 1)
    B = N.Field.from_numpy("XVol", b, 1)
    C = N.Field.from_numpy("XVol", c, 1)
    out, filt = N.Field("XVol", n, 1), N.Field("XVol", n, 1)
    words = N.mask_from_points(N.mask_words(out.glob), out.glob, 1, pts)
    N.deep_chain(A, B, C, words, out, filt)
    f2 = N.Field("XVol", n, 1)
    N.box_filter(out, f2)
    assert np.array_equal(filt.numpy().view(np.uint64), f2.numpy().view(np.uint64))
