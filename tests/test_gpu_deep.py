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
