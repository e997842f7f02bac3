"""Transposed stencil operators (nebo_stencil_transpose) and the FP32-forward gradient.

Each operator's dense Jacobian at 8^3 is built column by column from the oracle's forward
evaluation (the CPU restatement of the reference's stencil walk, spatialops/NeboStencils.h:407-448):
unit vector in, the written dst cells out.  The GPU transpose must equal J^T dst_bar on every
cell of src_bar's window (1e-14 relative: the gather sums the same products in another order),
written and accumulated.
"""
import numpy as np
import pytest

import oracle_dsl as O
import spatialops_gb300 as N
from spatialops_gb300 import workloads as W

pytestmark = pytest.mark.gpu

NN = (8, 8, 8)


def _operator(kind, src, dst):
    """(points, coefficients) of the forward operator as the oracle's operator table builds them."""
    db = O.OpDB(NN, (8.0, 6.0, 4.0))
    if kind == "interp":
        st = db.interp(src, dst)(O.Scalar(0.0))
    elif kind == "grad":
        st = db.grad(src, dst)(O.Scalar(0.0))
    elif kind == "div":
        st = db.div(src, dst)(O.Scalar(0.0))
    elif kind == "fdgrad":
        st = db.fd("grad", 0)(O.Scalar(0.0))
    else:  # the box filter's 27-point sum
        st = O.Stencil(O.OpDB.box_points(), None, O.Scalar(0.0))
    coefs = st.coefs if st.coefs is not None else [1.0] * len(st.pts)
    return st.pts, coefs, st.coefs is None


def _jacobian(pts, coefs, is_sum, src, dst, bc):
    gs, gd = O.glob_dims(src, NN, 1, bc), O.glob_dims(dst, NN, 1, bc)
    ns, nd = gs[0] * gs[1] * gs[2], gd[0] * gd[1] * gd[2]
    e = np.zeros(ns)
    S = O.Field(src, e.reshape(gs[2], gs[1], gs[0]), 1, bc)
    D = O.Field(dst, np.zeros((gd[2], gd[1], gd[0])), 1, bc)
    expr = O.Stencil(pts, None if is_sum else coefs, S)
    lim, _ = O.write_limits(D, expr)
    J = np.zeros((nd, ns))
    for j in range(ns):
        e[:] = 0.0
        e[j] = 1.0
        D.data[:] = 0.0
        O.assign(D, expr)
        J[:, j] = D.data.reshape(-1)
    # rows of cells outside the write region stay zero: the forward does not write them
    return J, lim


CASES = [
    ("interp", "SVol", "XVol", (0, 0, 0)),
    ("interp", "SVol", "YVol", (0, 0, 0)),
    ("grad", "SVol", "SSurfZ", (0, 0, 0)),
    ("div", "SSurfX", "SVol", (0, 0, 0)),
    ("interp", "XVol", "YVol", (0, 0, 0)),     # the four-point interpolant
    ("interp", "SVol", "XVol", (1, 0, 0)),     # with the +x boundary cell of XVol
    ("fdgrad", "SVol", "SVol", (0, 0, 0)),
    ("box", "SVol", "SVol", (0, 0, 0)),
]


@pytest.mark.parametrize("kind,src,dst,bc", CASES)
def test_stencil_transpose_equals_dense_jacobian_transpose(kind, src, dst, bc):
    pts, coefs, is_sum = _operator(kind, src, dst)
    J, lim = _jacobian(pts, coefs, is_sum, src, dst, bc)
    rng = np.random.default_rng(len(pts) * 7 + sum(bc))
    gd, gs = O.glob_dims(dst, NN, 1, bc), O.glob_dims(src, NN, 1, bc)
    dbar = rng.normal(size=(gd[2], gd[1], gd[0]))
    want = J.T @ dbar.reshape(-1)
    Dbar = N.Field.from_numpy(dst, dbar, 1, bc)
    Sbar = N.Field(src, NN, 1, bc)
    Sbar.tensor.fill_(123.0)  # overwritten everywhere
    N.stencil_transpose(Dbar, lim, Sbar, pts, coefs)
    got = Sbar.numpy().reshape(-1)
    scale = np.abs(J).sum(axis=0).max() * np.abs(dbar).max()
    assert np.abs(got - want).max() <= 1e-14 * scale, (kind, src, dst)
    # accumulate onto an existing value
    base = rng.normal(size=(gs[2], gs[1], gs[0]))
    Sbar2 = N.Field.from_numpy(src, base, 1, bc)
    N.stencil_transpose(Dbar, lim, Sbar2, pts, coefs, accumulate=True)
    assert np.abs(Sbar2.numpy().reshape(-1) - (base.reshape(-1) + want)).max() <= 1e-14 * (scale + np.abs(base).max())


def test_stencil_transpose_dot_product_identity_on_a_chain():
    """<Interp(Grad(a)), d> = <a, Grad^T(Interp^T(d))> for the deep chain's inner pair (XVol -> SVol
    -> XVol), composing the two transposes: the reverse mode of a nested stencil expression."""
    n = (24, 20, 16)
    db = O.OpDB(n, n)
    gi = db.grad("XVol", "SVol")(O.Scalar(0.0))
    ii = db.interp("SVol", "XVol")(O.Scalar(0.0))
    rng = np.random.default_rng(3)
    gx, gsv = O.glob_dims("XVol", n, 1, (0, 0, 0)), O.glob_dims("SVol", n, 1, (0, 0, 0))
    a = rng.normal(size=gx[::-1])
    A = O.Field("XVol", a, 1)
    mid = O.Field("SVol", np.zeros(gsv[::-1]), 1)
    lim1, _ = O.write_limits(mid, O.Stencil(gi.pts, gi.coefs, A))
    O.assign(mid, O.Stencil(gi.pts, gi.coefs, A))
    out = O.Field("XVol", np.zeros(gx[::-1]), 1)
    lim2, _ = O.write_limits(out, O.Stencil(ii.pts, ii.coefs, mid))
    O.assign(out, O.Stencil(ii.pts, ii.coefs, mid))
    d = rng.normal(size=gx[::-1])
    w = np.zeros(gx[::-1], dtype=bool)
    w[lim2[4] + 1:lim2[5] + 1, lim2[2] + 1:lim2[3] + 1, lim2[0] + 1:lim2[1] + 1] = True
    lhs = float((out.data * d)[w].sum())
    D = N.Field.from_numpy("XVol", d, 1)
    Mbar = N.Field("SVol", n, 1)
    N.stencil_transpose(D, lim2, Mbar, ii.pts, ii.coefs)
    Abar = N.Field("XVol", n, 1)
    # only the mid cells the first assignment wrote carry a value forward
    N.stencil_transpose(Mbar, lim1, Abar, gi.pts, gi.coefs)
    rhs = float((a * Abar.numpy()).sum())
    assert abs(lhs - rhs) <= 1e-12 * (abs(lhs) + 1.0), (lhs, rhs)


def test_gradient_with_fp32_forward_against_fp64():
    """nebo_heat_gradient_ex(NEBO_FORWARD_F32): FP32 forward states and checkpoints, FP64 adjoint.
    The gradient differs from the all-FP64 one by the FP32 rounding of the trajectory."""
    n, steps = (24, 20, 16), 40
    lam, T0, dt, lam_t = W.adjoint_inputs(n)
    Tt = O.heat_run(lam_t, T0, n, steps, dt)
    F = lambda a: N.Field.from_numpy("SVol", a, 1)
    J64, gT64, gl64 = N.heat_gradient(F(T0), F(lam), F(Tt), steps, dt)
    for every in (0, N.CHECKPOINT_AUTO):
        J32, gT32, gl32 = N.heat_gradient(F(T0), F(lam), F(Tt), steps, dt, every, forward="f32")
        I = (slice(1, -1),) * 3
        a, b = gT32.numpy()[I], gT64.numpy()[I]
        e_T = float(np.abs(a - b).max() / np.abs(b).max())
        c, d = gl32.numpy()[I], gl64.numpy()[I]
        e_l = float(np.abs(c - d).max() / np.abs(d).max())
        print(f"FP32 forward ({every}): dJ/dT0 rel err {e_T:.2e}, dJ/dlambda rel err {e_l:.2e}, "
              f"J rel diff {abs(J32 - J64) / J64:.2e}")
        assert e_T <= 1e-5 and e_l <= 1e-5
        assert abs(J32 - J64) <= 1e-5 * J64
