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


@pytest.mark.parametrize("n", [(64, 64, 64), (45, 30, 17)])
def test_deep_vs_oracle(n):
    a, b, c, pts = W.deep_inputs(n)
    out, filt, _ = _gpu(a, b, c, pts, n)
    o_out, o_filt = O.deep_run(a, b, c, W.mask_bits_from_points(pts, n), n)
    assert _relerr(out.numpy(), o_out) <= TOL
    assert _relerr(filt.numpy(), o_filt) <= TOL


@pytest.mark.parametrize("n,interior", [((64, 64, 64), False), ((45, 30, 17), False), ((45, 30, 17), True)])
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
