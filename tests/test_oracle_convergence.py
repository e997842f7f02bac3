"""The oracle's staggered operators against the reference's own convergence and filter tests
(spatialops/structured/stencil/test/test_stencil2.cpp: Interpolant, Gradient and Divergence
between a volume and its faces converge at second order in each direction; test_filter.cpp:
the box filter keeps a constant field).  A check of the operator table's points and
coefficients that does not go through golden vectors."""
import numpy as np
import pytest

import oracle_dsl as O

L = 10.0
K = 2.0 * np.pi / L


def _coord(loc, n, ghost, axis):
    """Coordinate along `axis` of every window point (cell centres at (i + 1/2) dx; a location
    staggered by -1/2 cell on an axis sits on the low faces)."""
    g = O.glob_dims(loc, n, ghost, (0, 0, 0))[axis]
    dx = L / n[axis]
    return (np.arange(g) - ghost + 0.5 + 0.5 * O.OFFSET[loc][axis]) * dx


def _field(loc, n, ghost, axis, fn):
    gdims = O.glob_dims(loc, n, ghost, (0, 0, 0))
    shape = (gdims[2], gdims[1], gdims[0])
    c = _coord(loc, n, ghost, axis)
    bshape = [1, 1, 1]
    bshape[2 - axis] = len(c)
    return np.broadcast_to(fn(c).reshape(bshape), shape).copy()


def _max_error(op, axis, N):
    n = [3, 3, 3]
    n[axis] = N
    n = tuple(n)
    ghost = 1
    db = O.OpDB(n, (L, L, L))
    face = ("SSurfX", "SSurfY", "SSurfZ")[axis]
    src, dst = ("SVol", face) if op != "div" else (face, "SVol")
    # source sin(K x); exact result sin(K x) (interpolant) or K cos(K x) (gradient, divergence)
    a = O.Field(src, _field(src, n, ghost, axis, lambda x: np.sin(K * x)), ghost)
    exact = (lambda x: np.sin(K * x)) if op == "interp" else (lambda x: K * np.cos(K * x))
    want = _field(dst, n, ghost, axis, exact)
    stencil = {"interp": db.interp, "grad": db.grad, "div": db.div}[op](src, dst)
    lhs = O.Field(dst, np.full_like(want, np.nan), ghost)
    O.assign(lhs, stencil(a), use_ghost=False)
    inner = (slice(ghost, -ghost),) * 3
    return float(np.max(np.abs(lhs.data[inner] - want[inner])))


@pytest.mark.parametrize("axis", [0, 1, 2])
@pytest.mark.parametrize("op", ["interp", "grad", "div"])
def test_second_order_convergence(op, axis):
    e = [_max_error(op, axis, N) for N in (16, 32, 64)]
    orders = [np.log2(e[i] / e[i + 1]) for i in range(2)]
    assert min(orders) > 1.9, (op, axis, e, orders)


def test_box_filter_keeps_constants():
    n, ghost = (9, 7, 5), 1
    db = O.OpDB(n, (L, L, L))
    g = O.glob_dims("SVol", n, ghost, (0, 0, 0))
    a = O.Field("SVol", np.full((g[2], g[1], g[0]), 3.25), ghost)
    lhs = O.Field("SVol", np.zeros((g[2], g[1], g[0])), ghost)
    O.assign(lhs, db.filter()(a), use_ghost=False)
    inner = (slice(ghost, -ghost),) * 3
    assert np.max(np.abs(lhs.data[inner] - 3.25)) <= 1e-15 * 3.25


def _field3(loc, n, ghost, fn):
    gd = O.glob_dims(loc, n, ghost, (0, 0, 0))
    cs = [_coord(loc, n, ghost, a) for a in range(3)]
    z, y, x = np.meshgrid(cs[2], cs[1], cs[0], indexing="ij")
    return np.ascontiguousarray(fn(x, y, z)).reshape(gd[2], gd[1], gd[0])


@pytest.mark.parametrize("src,dst", [("XVol", "YVol"), ("XVol", "ZVol"), ("YVol", "ZVol"), ("SSurfX", "SSurfY")])
def test_four_point_interpolant_second_order(src, dst):
    # the reference's test_stencil4.cpp: interpolants staggered in two directions (4 points, 1/4)
    fn = lambda x, y, z: np.sin(K * x) * np.cos(K * y) * np.sin(K * z + 0.3)
    e = []
    for N in (16, 32, 64):
        n, ghost = (N, N, N), 1
        db = O.OpDB(n, (L, L, L))
        assert len(db.stencil4_points(src, dst)) == 4
        a = O.Field(src, _field3(src, n, ghost, fn), ghost)
        want = _field3(dst, n, ghost, fn)
        lhs = O.Field(dst, np.full_like(want, np.nan), ghost)
        O.assign(lhs, db.interp(src, dst)(a), use_ghost=False)
        inner = (slice(ghost, -ghost),) * 3
        e.append(float(np.max(np.abs(lhs.data[inner] - want[inner]))))
    orders = [np.log2(e[i] / e[i + 1]) for i in range(2)]
    assert min(orders) > 1.9, (src, dst, e, orders)


def test_chained_stencils_equal_materialised():
    # the reference's test_chain_stencil.cpp: Interp(Grad(a)) evaluated in one assignment equals
    # the same two steps through a materialised intermediate field, bit for bit
    n, ghost = (11, 9, 7), 1
    db = O.OpDB(n, (L, 7.0, 5.0))
    rng = np.random.default_rng(3)
    gs = O.glob_dims("SVol", n, ghost, (0, 0, 0))
    a = O.Field("SVol", rng.uniform(-1, 1, (gs[2], gs[1], gs[0])), ghost)
    gx = O.glob_dims("SSurfX", n, ghost, (0, 0, 0))
    tmp = O.Field("SSurfX", np.full((gx[2], gx[1], gx[0]), np.nan), ghost)
    O.assign(tmp, db.grad("SVol", "SSurfX")(a))
    two = O.Field("SVol", np.full((gs[2], gs[1], gs[0]), np.nan), ghost)
    O.assign(two, db.interp("SSurfX", "SVol")(tmp))
    one = O.Field("SVol", np.full((gs[2], gs[1], gs[0]), np.nan), ghost)
    O.assign(one, db.interp("SSurfX", "SVol")(db.grad("SVol", "SSurfX")(a)))
    written = ~np.isnan(one.data)
    assert np.array_equal(written, ~np.isnan(two.data)) and written.any()
    assert np.array_equal(one.data[written].view(np.uint64), two.data[written].view(np.uint64))


def test_deep_chain_equals_stepwise():
    # the reference's test/StencilTestDeepChain.cpp: the deep chain
    #   out <<= cond(mask, 0)(I(G(I(a))) * exp(b) + sin(c))
    # evaluated in one assignment equals the same chain through materialised intermediates,
    # bit for bit, on every cell both write
    n, ghost = (10, 8, 6), 1
    db = O.OpDB(n, (L, 8.0, 6.0))
    rng = np.random.default_rng(5)

    def fld(loc, fill=None):
        g = O.glob_dims(loc, n, ghost, (0, 0, 0))
        data = rng.uniform(-1, 1, (g[2], g[1], g[0])) if fill is None else np.full((g[2], g[1], g[0]), fill)
        return O.Field(loc, data, ghost)

    a, b, c = fld("SVol"), fld("XVol"), fld("XVol")
    g = O.glob_dims("XVol", n, ghost, (0, 0, 0))
    pts = [(1, 1, 1), (3, 2, 0), (0, 0, 4), (7, 5, 2)]
    mask = O.Mask.from_points("XVol", pts, g, ghost)
    I1, G1, I2 = db.interp("SVol", "XVol"), db.grad("XVol", "SVol"), db.interp("SVol", "XVol")
    fused = fld("XVol", np.nan)
    O.assign(fused, O.cond(mask, 0.0, I2(G1(I1(a))) * O.exp(b) + O.sin(c)))
    t1, t2 = fld("XVol", np.nan), fld("SVol", np.nan)
    O.assign(t1, I1(a))
    O.assign(t2, G1(t1))
    t3 = fld("XVol", np.nan)
    O.assign(t3, I2(t2))
    step = fld("XVol", np.nan)
    O.assign(step, O.cond(mask, 0.0, t3 * O.exp(b) + O.sin(c)))
    both = ~np.isnan(fused.data) & ~np.isnan(step.data)
    assert both.sum() >= 0.5 * np.prod(n)
    assert np.array_equal(fused.data[both].view(np.uint64), step.data[both].view(np.uint64))
