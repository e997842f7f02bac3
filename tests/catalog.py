"""The expression catalog of tests/cpp/catalog_cases.inc, restated for the oracle.

run_catalog(domain) evaluates every case with the CPU restatement and returns records in the
same form as nebo_io.read_records, so they can be compared with the golden vectors that the
reference produced and with the GPU results of tests/cpp/catalog_gpu.cu.
"""
from __future__ import annotations

import numpy as np

import nebo_io
import oracle_dsl as O
from oracle_dsl import cond

DOMAINS = [
    dict(n=(7, 6, 5), ghost=1, bc=(0, 0, 0), L=(9.1, 5.4, 5.5)),
    dict(n=(6, 5, 4), ghost=1, bc=(1, 1, 1), L=(6.0, 6.5, 3.2)),
    dict(n=(6, 6, 6), ghost=2, bc=(0, 0, 0), L=(6.0, 7.2, 4.8)),
]


class Ctx:
    def __init__(self, domain):
        d = DOMAINS[domain]
        self.domain, self.n, self.ghost, self.bc = domain, d["n"], d["ghost"], d["bc"]
        self.db = O.OpDB(self.n, d["L"])
        self.inputs = {}
        self.records = {}

    def glob(self, loc):
        return O.glob_dims(loc, self.n, self.ghost, self.bc)

    def make(self, loc, values):
        g = self.glob(loc)
        return O.Field(loc, values.reshape(g[2], g[1], g[0]).copy(), self.ghost, self.bc)

    def inp(self, loc, k):
        key = (loc, k)
        if key not in self.inputs:
            g = self.glob(loc)
            v = nebo_io.uniform_pm1(nebo_io.field_stream(nebo_io.TYPE_CODES[loc], k, self.domain), g[0] * g[1] * g[2])
            self.inputs[key] = self.make(loc, v)
        return self.inputs[key]

    def fresh(self, loc):
        g = self.glob(loc)
        return self.make(loc, np.full(g[0] * g[1] * g[2], nebo_io.SENTINEL))

    def mask_points(self, k):
        return nebo_io.mask_points(k, self.domain, self.n, self.ghost)

    def mask(self, loc, k):
        return O.Mask.from_points(loc, self.mask_points(k), self.glob(loc), self.ghost, self.bc)

    def rec(self, name, f):
        self.records[name] = ("field", nebo_io.TYPE_CODES[f.loc], f.data)

    def val(self, name, v):
        self.records[name] = ("value", v)

    def case(self, name, fn):
        try:
            fn()
        except O.NeboError as e:
            self.records[name] = ("error", str(e))


def run_catalog(domain):
    C = Ctx(domain)
    db = C.db
    a, b, c = C.inp("SVol", 0), C.inp("SVol", 1), C.inp("SVol", 2)
    xa, xb, xc = C.inp("XVol", 0), C.inp("XVol", 1), C.inp("XVol", 2)

    def simple(name, loc, expr_fn, use_ghost=True):
        def body():
            out = C.fresh(loc)
            O.assign(out, expr_fn(), use_ghost)
            C.rec(name, out)
        C.case(name, body)

    # pointwise
    simple("s_copy", "SVol", lambda: a)
    simple("s_scalar", "SVol", lambda: O.Scalar(3.25))
    simple("s_add", "SVol", lambda: a + b)
    simple("s_sub", "SVol", lambda: a - b)
    simple("s_mul", "SVol", lambda: a * b)
    simple("s_div", "SVol", lambda: a / (b + 3.0))
    simple("s_scalar_mix", "SVol", lambda: 2.5 * a - b / 4.0 + 1.0 - (0.5 - c) * 3.0)
    simple("s_neg", "SVol", lambda: -a + -(b * c))
    simple("s_sin", "SVol", lambda: O.sin(a))
    simple("s_cos", "SVol", lambda: O.cos(a))
    simple("s_tan", "SVol", lambda: O.tan(a))
    simple("s_exp", "SVol", lambda: O.exp(a))
    simple("s_tanh", "SVol", lambda: O.tanh(a * 2.0))
    simple("s_abs", "SVol", lambda: O.abs_(a))
    simple("s_sqrt", "SVol", lambda: O.sqrt(O.abs_(a)))
    simple("s_log", "SVol", lambda: O.log(a * a + 0.5))
    simple("s_log10", "SVol", lambda: O.log10(O.abs_(b) + 0.25))
    simple("s_pow", "SVol", lambda: O.pow_(O.abs_(a) + 0.1, b))
    simple("s_powint", "SVol", lambda: O.pow_(a, 3))
    simple("s_square", "SVol", lambda: O.square(a) + O.cube(b))
    simple("s_maxmin", "SVol", lambda: O.max_(a, b) - O.min_(c, 0.25))

    # cond
    simple("s_cond_cmp", "SVol", lambda: cond(a > b, a, a < -0.5, b, c))
    simple("s_cond_logic", "SVol", lambda: cond((a > 0.0) & (b > 0.0), 1.0,
                                                (a <= 0.0) | ~(b < 0.5), 2.0,
                                                (a == a) & (b != c), 3.0, 4.0))
    simple("s_cond_ge", "SVol", lambda: cond(a >= 0.25, a * 2.0, b))

    # masks
    simple("s_cond_mask", "SVol", lambda: cond(C.mask("SVol", 0), a, C.mask("SVol", 1), 7.0, b))
    simple("s_cond_mask_logic", "SVol",
           lambda: cond(C.mask("SVol", 0) | C.mask("SVol", 1), 1.0,
                        ~C.mask("SVol", 0) & (a > 0.0), 2.0, 3.0))

    def masked():
        out = C.fresh("SVol")
        O.masked_assign(C.mask_points(0), out, a * b)
        C.rec("s_masked_assign", out)
    C.case("s_masked_assign", masked)
    simple("s_interior", "SVol", lambda: a + 2.0 * b, use_ghost=False)

    # SVol basic operator types
    fx, fy, fz = O.FACES["SVol"]
    simple("s_interpc2fx", fx, lambda: db.interp("SVol", fx)(a))
    simple("s_interpc2fy", fy, lambda: db.interp("SVol", fy)(a))
    simple("s_interpc2fz", fz, lambda: db.interp("SVol", fz)(a))
    simple("s_gradx", fx, lambda: db.grad("SVol", fx)(a))
    simple("s_grady", fy, lambda: db.grad("SVol", fy)(a))
    simple("s_gradz", fz, lambda: db.grad("SVol", fz)(a))
    simple("s_divx", "SVol", lambda: db.div(fx, "SVol")(C.inp(fx, 0)))
    simple("s_divy", "SVol", lambda: db.div(fy, "SVol")(C.inp(fy, 0)))
    simple("s_divz", "SVol", lambda: db.div(fz, "SVol")(C.inp(fz, 0)))
    simple("s_interpf2cx", "SVol", lambda: db.interp(fx, "SVol")(C.inp(fx, 1)))
    simple("s_interpf2cy", "SVol", lambda: db.interp(fy, "SVol")(C.inp(fy, 1)))
    simple("s_interpf2cz", "SVol", lambda: db.interp(fz, "SVol")(C.inp(fz, 1)))

    # staggered volume <-> scalar volume
    simple("s2x_interp", "XVol", lambda: db.interp("SVol", "XVol")(a))
    simple("s2y_grad", "YVol", lambda: db.grad("SVol", "YVol")(a))
    simple("s2z_interp", "ZVol", lambda: db.interp("SVol", "ZVol")(b))
    simple("x2s_grad", "SVol", lambda: db.grad("XVol", "SVol")(xa))
    simple("y2s_interp", "SVol", lambda: db.interp("YVol", "SVol")(C.inp("YVol", 0)))
    simple("z2s_grad", "SVol", lambda: db.grad("ZVol", "SVol")(C.inp("ZVol", 0)))

    # XVol basic operator types
    xfx, xfy, xfz = O.FACES["XVol"]
    simple("x_gradx", xfx, lambda: db.grad("XVol", xfx)(xa))
    simple("x_interpc2fy", xfy, lambda: db.interp("XVol", xfy)(xa))
    simple("x_divz", "XVol", lambda: db.div(xfz, "XVol")(C.inp(xfz, 0)))

    # 4-point interpolants
    simple("s2xsurfy_interp4", "XSurfY", lambda: db.interp("SVol", "XSurfY")(a))
    simple("s2zsurfx_interp4", "ZSurfX", lambda: db.interp("SVol", "ZSurfX")(b))
    simple("x2y_interp4", "YVol", lambda: db.interp("XVol", "YVol")(xa))
    simple("x2z_interp4", "ZVol", lambda: db.interp("XVol", "ZVol")(xb))

    # null interpolants
    simple("x2ssurfx_null", "SSurfX", lambda: db.interp("XVol", "SSurfX")(xa))
    simple("s_null", "SVol", lambda: db.interp("SVol", "SVol")(a))

    # finite-difference stencils
    simple("s_fd_gradx", "SVol", lambda: db.fd("grad", 0)(a))
    simple("s_fd_grady", "SVol", lambda: db.fd("grad", 1)(a))
    simple("s_fd_interpz", "SVol", lambda: db.fd("interp", 2)(a))
    simple("x_fd_gradz", "XVol", lambda: db.fd("grad", 2)(xa))
    simple("s_user_pair", "SVol", lambda: O.Stencil([(0, 0, 0), (1, 0, 0)], [0.25, 0.75], a) * b)

    # box filter
    simple("s_filter", "SVol", lambda: db.filter()(a))
    simple("x_filter", "XVol", lambda: db.filter()(xa))

    # chains
    is2x, gx2s, box = db.interp("SVol", "XVol"), db.grad("XVol", "SVol"), db.filter()
    simple("chain_igi", "XVol", lambda: is2x(gx2s(is2x(a))))

    def deep():
        m = C.mask("XVol", 0)
        out = C.fresh("XVol")
        O.assign(out, O.Scalar(0.0))
        O.assign(out, cond(m, 0.0, is2x(gx2s(is2x(a))) * O.exp(xb) + O.sin(xc)))
        f = C.fresh("XVol")
        O.assign(f, box(out))
        C.rec("chain_deep_out", out)
        C.rec("chain_deep_filt", f)
        C.val("chain_deep_sum", O.reduce("sum", f))
        C.val("chain_deep_max", O.reduce("max", f))
        C.val("chain_deep_norm", O.reduce("norm", f))
    C.case("chain_deep", deep)

    def heat_rhs():
        ix, iy, iz = (db.interp("SVol", f) for f in (fx, fy, fz))
        gx, gy, gz = (db.grad("SVol", f) for f in (fx, fy, fz))
        dx, dy, dz = (db.div(f, "SVol") for f in (fx, fy, fz))
        return a + 0.05 * (dx(ix(b) * gx(a)) + dy(iy(b) * gy(a)) + dz(iz(b) * gz(a)))
    simple("chain_heat_rhs", "SVol", heat_rhs)
    simple("chain_filter_cond", "SVol", lambda: db.filter()(cond(a > 0.0, a, b * 0.5)))

    # SingleValue fields (catalog_ctx.h: 2u + 0.25 in a 1x1x1 window): in an expression the value
    # with no ghost limit, which the oracle's scalar leaf is; SingleValue results are 1x1x1 records
    def sv(k):
        return 2.0 * float(nebo_io.uniform_pm1(nebo_io.field_stream(17, k, C.domain), 1)[0]) + 0.25
    s1, s2 = sv(0), sv(1)
    S1, S2 = O.Scalar(s1), O.Scalar(s2)

    def sv_rec(name, v):
        C.records[name] = ("field", nebo_io.TYPE_CODES["SingleValue"], np.full((1, 1, 1), v, dtype=np.float64))

    simple("sv_broadcast", "SVol", lambda: S1)
    simple("sv_times_int", "SVol", lambda: S1 * 4.0)
    simple("sv_minus_field", "SVol", lambda: S1 - a)
    simple("sv_div_sv", "SVol", lambda: S1 / S2)
    simple("sv_mixed", "XVol", lambda: xa * (S1 + S2) - S2 * 0.5)
    sv_rec("sv_to_sv", s1 * s2 + 1.5)
    sv_rec("sv_copy", s2)
    sv_rec("sv_scalar", 2.75)
    simple("sv_interior", "SVol", lambda: S1 + 0.25, use_ghost=False)
    simple("sv_stencil", "XVol", lambda: is2x(a) * S1 + S2)
    simple("cond_final_sv", "SVol", lambda: S1 + S2)
    simple("cond_final_field", "SVol", lambda: a + b)
    simple("cond_bool_sv", "SVol", lambda: O.Scalar(2.0))  # cond(false, sv1)(2.0)
    simple("cond_bool_field", "SVol", lambda: a + b)       # cond(true, a + b)(2.0)
    simple("cond_sv_test", "SVol", lambda: cond(S1 < 0.0, a, S2 * 2.0))
    sv_rec("cond_sv_to_sv", s1 + s2 if s1 > s2 else s2)
    simple("cond_field_sv_value", "SVol", lambda: cond(a > 0.0, S1, b))
    C.val("cond_simple", 1.0 + 10.0 * 2.0 + 100.0 * 4.5)

    # reductions
    def red_field():
        for op in ("sum", "max", "min", "norm"):
            C.val("red_" + op, O.reduce(op, a))
        for op in ("sum", "max", "min", "norm"):
            C.val(f"red_{op}_interior", O.reduce(op, a, interior=True))
    C.case("red_field", red_field)

    def red_expr():
        C.val("red_expr_sum", O.reduce("sum", a * b + c))
        C.val("red_expr_max", O.reduce("max", O.sin(a) - b))
        C.val("red_expr_norm_interior", O.reduce("norm", a - b, interior=True))
    C.case("red_expr", red_expr)

    def red_x():
        C.val("red_x_sum", O.reduce("sum", xa))
        C.val("red_x_max_interior", O.reduce("max", xb, interior=True))
    C.case("red_xvol", red_x)

    # apply_pointwise: the operands evaluated by the oracle, the functor in IEEE double (numpy,
    # element-wise, no contraction) over the write region the operands' ghosts allow
    def apply_case(name, fn, ops):
        def body():
            out = C.fresh("SVol")
            lim, ok = O.write_limits(out, sum(o for o in ops if not isinstance(o, float)))
            if not ok:
                raise O.NeboError("write limits")
            vals = []
            for o in ops:
                if isinstance(o, float):
                    vals.append(o)
                    continue
                f = C.fresh("SVol")
                O.assign(f, o)
                vals.append(f.data)
            g = out.ghost
            sl = tuple(slice(lim[2 * i] + g, lim[2 * i + 1] + g) for i in (2, 1, 0))
            args = [v if isinstance(v, float) else v[sl] for v in vals]
            out.data[sl] = fn(*args)
            C.rec(name, out)
        C.case(name, body)

    apply_case("s_apply_sum4", lambda i1, i2, i3, i4: i1 + i2 + i3 + i4, [a + b, c, 5.0, 6.0])
    apply_case("s_apply_quad", lambda v: v * v - 3.0, [a * b])
    apply_case("s_apply_mix7_stencil", lambda a_, b_, c_, d_, e_, f_, g_: (a_ * b_ - c_) / (d_ + 2.5) + e_ * f_ - g_,
               [a, b, c, db.fd("grad", 0)(a), 1.5, b * c, a - 1.0])

    # boundary conditions (NeboBoundaryConditionBuilder over whole boundary planes)
    n = C.n

    def plane(axis, i):
        a1, a2 = (axis + 1) % 3, (axis + 2) % 3
        pts = []
        for v in range(n[a2]):
            for u in range(n[a1]):
                q = [0, 0, 0]
                q[axis], q[a1], q[a2] = i, u, v
                pts.append(tuple(q))
        return pts

    def evaluated(loc, expr):
        f = C.fresh(loc)
        O.assign(f, expr)
        return O.field_values(f)

    def stencil(builder):
        st = builder(a)
        return st.pts, st.coefs

    def copy_of(loc, src):
        f = C.fresh(loc)
        O.assign(f, src)
        return f

    def bc_gradx():
        pts, cf = stencil(db.grad("SVol", "SSurfX"))
        phi = copy_of("SVol", a)
        O.bc_apply(phi, O.field_values(C.inp("SSurfX", 0)), plane(0, 0),
                   O.bc_geometry(pts, cf, "SVol", "SSurfX", True))
        O.bc_apply(phi, lambda x, y, z: 0.75, plane(0, n[0]), O.bc_geometry(pts, cf, "SVol", "SSurfX", False))
        C.rec("bc_gradx_field_and_scalar", phi)
    C.case("bc_gradx_field_and_scalar", bc_gradx)

    def bc_interpy():
        pts, cf = stencil(db.interp("SVol", "SSurfY"))
        phi = copy_of("SVol", b)
        gy = C.inp("SSurfY", 1)
        O.bc_apply(phi, evaluated("SSurfY", gy * gy * 2.0 + 1.0), plane(1, 0),
                   O.bc_geometry(pts, cf, "SVol", "SSurfY", True))
        O.bc_apply(phi, evaluated("SSurfY", gy - 0.5), plane(1, n[1]),
                   O.bc_geometry(pts, cf, "SVol", "SSurfY", False))
        C.rec("bc_interpy_expr", phi)
    C.case("bc_interpy_expr", bc_interpy)

    def bc_divz():
        st = db.div("SSurfZ", "SVol")(C.inp("SSurfZ", 2))
        pts, cf = st.pts, st.coefs
        phi = copy_of("SSurfZ", C.inp("SSurfZ", 2))
        O.bc_apply(phi, O.field_values(c), plane(2, n[2] - 1), O.bc_geometry(pts, cf, "SSurfZ", "SVol", False))
        O.bc_apply(phi, lambda x, y, z: 1.25, plane(2, 0), O.bc_geometry(pts, cf, "SSurfZ", "SVol", True))
        C.rec("bc_divz_faces", phi)
    C.case("bc_divz_faces", bc_divz)

    def bc_fd():
        pts, cf = stencil(db.fd("grad", 0))
        phi = copy_of("SVol", c)
        O.bc_apply(phi, O.field_values(a), plane(0, 0), O.bc_geometry(pts, cf, "SVol", "SVol", True, (1, 0, 0)))
        O.bc_apply(phi, evaluated("SVol", b * 2.0), plane(0, n[0] - 1),
                   O.bc_geometry(pts, cf, "SVol", "SVol", False, (1, 0, 0)))
        C.rec("bc_fd_gradx", phi)
    C.case("bc_fd_gradx", bc_fd)
    return C.records
