"""Python front end of the oracle (oracle/nebo_oracle.cpp) for the tests.

Builds Nebo-like expression trees in Python, encodes them in the oracle's prefix program and
evaluates them with the CPU restatement.  The location-type table, stencil point collections
and coefficients restate the reference's:
  spatialops/structured/FVStaggeredLocationTypes.h:63-126   (offsets, BCExtra)
  spatialops/structured/FVStaggeredFieldTypes.h:148-217     (FaceTypes)
  spatialops/NeboStencilBuilder.h:154-232, 454-501          (Stencil2/4, FD, box filter points)
  spatialops/structured/stencil/StencilBuilder.cpp:52-220   (coefficients)
  spatialops/structured/MemoryWindow.h:290-321              (glob dims with ghosts and BC cells)
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE_SO = os.path.join(REPO, "oracle", "_build", "liboracle.so")

# ----------------------------------------------------------------------------- locations
OFFSET = {
    "SVol": (0, 0, 0), "SSurfX": (-1, 0, 0), "SSurfY": (0, -1, 0), "SSurfZ": (0, 0, -1),
    "XVol": (-1, 0, 0), "XSurfX": (0, 0, 0), "XSurfY": (-1, -1, 0), "XSurfZ": (-1, 0, -1),
    "YVol": (0, -1, 0), "YSurfX": (-1, -1, 0), "YSurfY": (0, 0, 0), "YSurfZ": (0, -1, -1),
    "ZVol": (0, 0, -1), "ZSurfX": (-1, 0, -1), "ZSurfY": (0, -1, -1), "ZSurfZ": (0, 0, 0),
}
BCEXTRA = {
    "SVol": (0, 0, 0), "SSurfX": (1, 0, 0), "SSurfY": (0, 1, 0), "SSurfZ": (0, 0, 1),
    "XVol": (1, 0, 0), "XSurfX": (0, 0, 0), "XSurfY": (0, 1, 0), "XSurfZ": (0, 0, 1),
    "YVol": (0, 1, 0), "YSurfX": (1, 0, 0), "YSurfY": (0, 0, 0), "YSurfZ": (0, 0, 1),
    "ZVol": (0, 0, 1), "ZSurfX": (1, 0, 0), "ZSurfY": (0, 1, 0), "ZSurfZ": (0, 0, 0),
}
FACES = {
    "SVol": ("SSurfX", "SSurfY", "SSurfZ"), "XVol": ("XSurfX", "XSurfY", "XSurfZ"),
    "YVol": ("YSurfX", "YSurfY", "YSurfZ"), "ZVol": ("ZSurfX", "ZSurfY", "ZSurfZ"),
}


def glob_dims(loc, n, ghost, bc):
    ex = BCEXTRA[loc]
    return tuple((n[i] + 2 * ghost + (ex[i] if bc[i] else 0)) if n[i] > 1 else 1 for i in range(3))


# ----------------------------------------------------------------------------- library
class _Field(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("glob", ctypes.c_int32 * 3), ("ghost_minus", ctypes.c_int32 * 3),
                ("ghost_plus", ctypes.c_int32 * 3), ("has_bc", ctypes.c_int32 * 3), ("bc_extra", ctypes.c_int32 * 3)]


class _Mask(ctypes.Structure):
    _fields_ = [("bits", ctypes.c_void_p), ("glob", ctypes.c_int32 * 3), ("ghost_minus", ctypes.c_int32 * 3),
                ("ghost_plus", ctypes.c_int32 * 3), ("has_bc", ctypes.c_int32 * 3), ("bc_extra", ctypes.c_int32 * 3)]


class _Expr(ctypes.Structure):
    _fields_ = [("prog", ctypes.c_void_p), ("prog_len", ctypes.c_int32), ("imms", ctypes.c_void_p),
                ("fields", ctypes.c_void_p), ("nfields", ctypes.c_int32), ("masks", ctypes.c_void_p),
                ("nmasks", ctypes.c_int32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            subprocess.run(["make", "-C", os.path.join(REPO, "oracle"), "liboracle"], check=True,
                           stdout=subprocess.DEVNULL)
        _lib = ctypes.CDLL(ORACLE_SO)
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


# ----------------------------------------------------------------------------- expression tree
class E:
    def __add__(self, o): return Bin(0, self, lift(o))
    def __radd__(self, o): return Bin(0, lift(o), self)
    def __sub__(self, o): return Bin(1, self, lift(o))
    def __rsub__(self, o): return Bin(1, lift(o), self)
    def __mul__(self, o): return Bin(2, self, lift(o))
    def __rmul__(self, o): return Bin(2, lift(o), self)
    def __truediv__(self, o): return Bin(3, self, lift(o))
    def __rtruediv__(self, o): return Bin(3, lift(o), self)
    def __neg__(self): return Un(0, self)
    def __eq__(self, o): return Cmp(0, self, lift(o))
    def __ne__(self, o): return Cmp(1, self, lift(o))
    def __lt__(self, o): return Cmp(2, self, lift(o))
    def __le__(self, o): return Cmp(3, self, lift(o))
    def __gt__(self, o): return Cmp(4, self, lift(o))
    def __ge__(self, o): return Cmp(5, self, lift(o))
    def __and__(self, o): return Logic(0, self, o)
    def __or__(self, o): return Logic(1, self, o)
    def __invert__(self): return Logic(2, self)
    __hash__ = object.__hash__


def lift(v):
    return v if isinstance(v, E) else Scalar(float(v))


class Scalar(E):
    def __init__(self, v): self.v = v
    def enc(self, c): c.prog += [2, c.imm(self.v)]


class Field(E):
    """A field leaf over a numpy (gz, gy, gx) float64 window."""

    def __init__(self, loc, data, ghost, bc=(0, 0, 0)):
        self.loc, self.data, self.ghost, self.bc = loc, data, ghost, tuple(bc)

    def enc(self, c): c.prog += [1, c.field(self)]

    def desc(self):
        d = _Field()
        d.data = self.data.ctypes.data
        gz, gy, gx = self.data.shape
        d.glob[:] = (gx, gy, gz)
        d.ghost_minus[:] = (self.ghost,) * 3
        d.ghost_plus[:] = (self.ghost,) * 3
        d.has_bc[:] = self.bc
        d.bc_extra[:] = BCEXTRA[self.loc]
        return d


class Mask(E):
    def __init__(self, loc, bits, glob, ghost, bc=(0, 0, 0)):
        self.loc, self.bits, self.glob, self.ghost, self.bc = loc, bits, glob, ghost, tuple(bc)

    @staticmethod
    def from_points(loc, pts, glob, ghost, bc=(0, 0, 0)):
        bits = np.zeros((glob[0] * glob[1] * glob[2] + 31) // 32 + 1, dtype=np.uint32)
        g3 = (ctypes.c_int32 * 3)(*glob)
        off = (ctypes.c_int32 * 3)(ghost, ghost, ghost)
        pts = np.ascontiguousarray(pts, dtype=np.int32)
        lib().orc_mask_from_points(_p(bits), g3, off, _p(pts), ctypes.c_int(len(pts)))
        return Mask(loc, bits, glob, ghost, bc)

    def enc(self, c): c.prog += [9, c.mask(self)]

    def desc(self):
        d = _Mask()
        d.bits = self.bits.ctypes.data
        d.glob[:] = self.glob
        d.ghost_minus[:] = (self.ghost,) * 3
        d.ghost_plus[:] = (self.ghost,) * 3
        d.has_bc[:] = self.bc
        d.bc_extra[:] = BCEXTRA[self.loc]
        return d


class Bin(E):
    def __init__(self, op, a, b): self.op, self.a, self.b = op, a, b
    def enc(self, c): c.prog += [3, self.op]; self.a.enc(c); self.b.enc(c)


class Un(E):
    def __init__(self, fn, a): self.fn, self.a = fn, a
    def enc(self, c): c.prog += [4, self.fn]; self.a.enc(c)


class PowInt(E):
    def __init__(self, a, e): self.a, self.e = a, e
    def enc(self, c): c.prog += [5, self.e]; self.a.enc(c)


class Cmp(E):
    def __init__(self, op, a, b): self.op, self.a, self.b = op, a, b
    def enc(self, c): c.prog += [6, self.op]; self.a.enc(c); self.b.enc(c)


class Logic(E):
    def __init__(self, op, a, b=None): self.op, self.a, self.b = op, a, b

    def enc(self, c):
        c.prog += [7, self.op]
        self.a.enc(c)
        if self.b is not None:
            self.b.enc(c)


class Cond(E):
    def __init__(self, clauses, default): self.clauses, self.default = clauses, lift(default)

    def enc(self, c):
        c.prog += [8, len(self.clauses)]
        for t, v in self.clauses:
            t.enc(c)
            lift(v).enc(c)
        self.default.enc(c)


def cond(*args):
    """cond(t0, v0, t1, v1, ..., default)."""
    pairs = [(args[i], args[i + 1]) for i in range(0, len(args) - 1, 2)]
    return Cond(pairs, args[-1])


class Stencil(E):
    def __init__(self, pts, coefs, arg):
        self.pts, self.coefs, self.arg = [tuple(p) for p in pts], coefs, lift(arg)

    def enc(self, c):
        if self.coefs is None:
            c.prog += [11, len(self.pts)]
            for p in self.pts:
                c.prog += list(p)
        else:
            c.prog += [10, len(self.pts)]
            for p in self.pts:
                c.prog += list(p)
            c.prog.append(c.imms_block(self.coefs))
        self.arg.enc(c)


def _fn(code):
    return lambda a: Un(code, lift(a))


sin, cos, tan, exp, tanh, abs_, sqrt, log, log10, erf, erfc, square, cube = (
    _fn(i) for i in range(1, 14))


def pow_(a, b):
    if isinstance(b, int):
        return PowInt(lift(a), b)
    return Bin(4, lift(a), lift(b))


def max_(a, b): return Bin(5, lift(a), lift(b))
def min_(a, b): return Bin(6, lift(a), lift(b))


class _Enc:
    def __init__(self):
        self.prog, self.imms, self.fields, self.masks = [], [], [], []

    def imm(self, v):
        self.imms.append(float(v))
        return len(self.imms) - 1

    def imms_block(self, vs):
        i = len(self.imms)
        self.imms += [float(v) for v in vs]
        return i

    def field(self, f):
        for i, g in enumerate(self.fields):
            if g is f:
                return i
        self.fields.append(f)
        return len(self.fields) - 1

    def mask(self, m):
        for i, g in enumerate(self.masks):
            if g is m:
                return i
        self.masks.append(m)
        return len(self.masks) - 1


class _Compiled:
    def __init__(self, e):
        c = _Enc()
        lift(e).enc(c)
        self.prog = np.array(c.prog, dtype=np.int32)
        self.imms = np.array(c.imms + [0.0], dtype=np.float64)
        self.fdesc = (_Field * max(1, len(c.fields)))(*[f.desc() for f in c.fields])
        self.mdesc = (_Mask * max(1, len(c.masks)))(*[m.desc() for m in c.masks])
        self.keep = (c.fields, c.masks)
        self.e = _Expr(self.prog.ctypes.data, len(self.prog), self.imms.ctypes.data,
                       ctypes.cast(self.fdesc, ctypes.c_void_p), len(c.fields),
                       ctypes.cast(self.mdesc, ctypes.c_void_p), len(c.masks))


class NeboError(RuntimeError):
    pass


def _check(rc, err):
    if rc == 1:
        raise NeboError(err.value.decode())
    return rc


def assign(lhs: Field, expr, use_ghost=True):
    """lhs <<= expr (use_ghost=False: interior_assign)."""
    comp = _Compiled(expr)
    err = ctypes.create_string_buffer(512)
    d = lhs.desc()
    _check(lib().orc_assign(ctypes.byref(comp.e), ctypes.byref(d), int(use_ghost), err, 512), err)
    return lhs


def write_limits(lhs: Field, expr, use_ghost=True):
    comp = _Compiled(expr)
    err = ctypes.create_string_buffer(512)
    lim = (ctypes.c_int32 * 6)()
    d = lhs.desc()
    rc = _check(lib().orc_write_limits(ctypes.byref(comp.e), ctypes.byref(d), int(use_ghost), lim, err, 512), err)
    return tuple(lim), rc == 0


def masked_assign(points, lhs: Field, expr):
    comp = _Compiled(expr)
    err = ctypes.create_string_buffer(512)
    pts = np.ascontiguousarray(points, dtype=np.int32)
    d = lhs.desc()
    _check(lib().orc_masked_assign(ctypes.byref(comp.e), ctypes.byref(d), _p(pts), len(pts), err, 512), err)
    return lhs


def bc_geometry(pts, coefs, phi_loc, gamma_loc, minus, fd_dir=None):
    """NeboBoundaryConditionBuilder's geometry (spatialops/NeboStencilBuilder.h:503-526,584-640)
    for a stencil with points `pts` / coefficients `coefs` in listed order (first listed = Low,
    last listed = High):
      minus: gamma point -Low, phi points pts[1:] - Low with coefs[1:], divisor coefs[0];
      plus:  gamma point -High, phi points pts[:-1] - High with coefs[:-1], divisor coefs[-1];
      mask shift: for two location types, minus = (gamma offset < phi offset) per axis and
      plus = -(gamma offset > phi offset); for one type (FD) +-the stencil direction.
    Returns (shift, gamma_point, phi_points, phi_coefs, divisor)."""
    sub = lambda p, q: tuple(p[i] - q[i] for i in range(3))
    if minus:
        piv, gpt, rest, rc, div = pts[0], None, pts[1:], coefs[1:], coefs[0]
    else:
        piv, gpt, rest, rc, div = pts[-1], None, pts[:-1], coefs[:-1], coefs[-1]
    gpt = tuple(-v for v in piv)
    if phi_loc == gamma_loc:
        shift = tuple(fd_dir) if minus else tuple(-v for v in fd_dir)
    else:
        go, po = OFFSET[gamma_loc], OFFSET[phi_loc]
        shift = tuple(1 if go[i] < po[i] else 0 for i in range(3)) if minus else \
            tuple(-(1 if go[i] > po[i] else 0) for i in range(3))
    return shift, gpt, [sub(q, piv) for q in rest], list(rc), div


def bc_apply(phi: Field, gamma_value, points, geometry):
    """The reference's serial BC point loop (NeboBoundaryConditionBuilder::cpu_apply,
    spatialops/NeboStencilBuilder.h:641-678): for every mask point m, p = m - shift and
      phi[p] = (1.0 * gamma[p + gamma_point] - fold_q c_q phi[p + q]) / divisor
    with the stencil fold of NeboStencils.h:415-440 (first point first), in IEEE double, in
    point order.  gamma_value(x, y, z) returns the gamma expression at a gamma-field index."""
    shift, gpt, qs, cs, div = geometry
    g = phi.ghost
    at = lambda x, y, z: (z + g, y + g, x + g)
    for m in points:
        p = tuple(int(m[i]) - shift[i] for i in range(3))
        s = None
        for q, c in zip(qs, cs):
            term = float(c) * float(phi.data[at(p[0] + q[0], p[1] + q[1], p[2] + q[2])])
            s = term if s is None else s + term
        gv = 1.0 * float(gamma_value(p[0] + gpt[0], p[1] + gpt[1], p[2] + gpt[2]))
        phi.data[at(*p)] = (gv - s) / float(div)
    return phi


def field_values(f: Field):
    """Callable (x, y, z) -> f at that interior-relative index (ghosts included)."""
    g = f.ghost
    return lambda x, y, z: f.data[z + g, y + g, x + g]


RED = {"sum": 0, "max": 1, "min": 2, "norm": 3}


def reduce(op, expr, interior=False):
    comp = _Compiled(expr)
    err = ctypes.create_string_buffer(512)
    out = ctypes.c_double()
    _check(lib().orc_reduce(ctypes.byref(comp.e), RED[op], int(not interior), ctypes.byref(out), err, 512), err)
    return out.value


# ----------------------------------------------------------------------------- operator table
class OpDB:
    """build_stencils(nx, ny, nz, Lx, Ly, Lz): returns stencil builders by (op, src, dest)."""

    def __init__(self, n, L):
        self.dx = [L[i] / n[i] for i in range(3)]

    @staticmethod
    def _gt(a, b): return tuple(1 if a[i] > b[i] else 0 for i in range(3))

    @staticmethod
    def _lt(a, b): return tuple(1 if a[i] < b[i] else 0 for i in range(3))

    def stencil2_points(self, src, dest):
        so, do = OFFSET[src], OFFSET[dest]
        low = tuple(-v for v in self._gt(so, do))
        high = self._lt(so, do)
        return [low, high]

    def stencil4_points(self, src, dest):
        so, do = OFFSET[src], OFFSET[dest]
        first = (1, 0, 0) if so[0] != do[0] else (0, 1, 0)
        second = (0, 0, 1) if so[2] != do[2] else (0, 1, 0)
        mul = lambda a, b: tuple(a[i] * b[i] for i in range(3))
        add = lambda a, b: tuple(a[i] + b[i] for i in range(3))
        sf, ss, df, ds = mul(so, first), mul(so, second), mul(do, first), mul(do, second)
        lo1 = tuple(-v for v in self._gt(sf, df))
        hi1 = self._lt(sf, df)
        lo2 = tuple(-v for v in self._gt(ss, ds))
        hi2 = self._lt(ss, ds)
        return [add(lo1, lo2), add(hi1, lo2), add(lo1, hi2), add(hi1, hi2)]

    def _grad_axis(self, src, dest):
        so, do = OFFSET[src], OFFSET[dest]
        for i in range(3):
            if so[i] != do[i]:
                return i
        raise ValueError("no staggering direction")

    def interp(self, src, dest):
        if OFFSET[src] == OFFSET[dest]:
            return lambda a: Stencil([(0, 0, 0)], None, a)  # null stencil (sum of one point)
        pts = self.stencil2_points(src, dest) if self._nstag(src, dest) == 1 else self.stencil4_points(src, dest)
        coefs = [0.5, 0.5] if len(pts) == 2 else [0.25] * 4
        return lambda a: Stencil(pts, coefs, a)

    @staticmethod
    def _nstag(src, dest):
        return sum(1 for i in range(3) if OFFSET[src][i] != OFFSET[dest][i])

    def grad(self, src, dest):
        """Gradient (and Divergence, which shares the 2-point shape and coefficients)."""
        ax = self._grad_axis(src, dest)
        pts = self.stencil2_points(src, dest)
        d = self.dx[ax]
        return lambda a: Stencil(pts, [-1.0 / d, 1.0 / d], a)

    div = grad

    def fd(self, kind, axis):
        unit = [0, 0, 0]
        unit[axis] = 1
        pts = [tuple(-u for u in unit), tuple(unit)]
        if kind == "interp":
            return lambda a: Stencil(pts, [0.5, 0.5], a)
        d = self.dx[axis]
        return lambda a: Stencil(pts, [-0.5 / d, 0.5 / d], a)

    @staticmethod
    def box_points():
        return [(x, y, z) for z in (-1, 0, 1) for y in (-1, 0, 1) for x in (-1, 0, 1)]

    def filter(self):
        pts = self.box_points()
        return lambda a: Stencil(pts, None, a) * (1.0 / 27.0)


# ----------------------------------------------------------------------------- workload drivers
def _i3(v):
    return (ctypes.c_int32 * 3)(*v)


def heat_run(lam, T0, n, steps, dt, threads=1):
    """Returns T after `steps` Euler steps (full window, ghosts periodic)."""
    T = np.ascontiguousarray(T0, dtype=np.float64).copy()
    tmp = np.zeros_like(T)
    lam = np.ascontiguousarray(lam, dtype=np.float64)
    lib().orc_heat_run(_p(T), _p(tmp), _p(lam), _i3(n), int(steps), ctypes.c_double(dt), int(threads))
    return T


def deep_run(a, b, c, maskbits, n, dx=1.0, threads=1):
    out = np.empty_like(b)
    filt = np.empty_like(b)
    lib().orc_deep_run(_p(a), _p(b), _p(c), _p(maskbits), _p(out), _p(filt), _i3(n), ctypes.c_double(dx),
                       int(threads))
    return out, filt


def deep_write_region(n, ghost=1):
    """The write region of out <<= cond(mask, 0)(I(G(I(a))) * exp(b) + sin(c)) as write_limits
    returns it, by the oracle's restatement of calculate_actual_ghost (host integer code; the
    fields are zero-stride stand-ins, never read)."""
    gs, gx = glob_dims("SVol", n, ghost, (0, 0, 0)), glob_dims("XVol", n, ghost, (0, 0, 0))
    one = np.empty(1)
    a = Field("SVol", np.lib.stride_tricks.as_strided(one, shape=gs[::-1], strides=(0, 0, 0)), ghost)
    bx = np.lib.stride_tricks.as_strided(one, shape=gx[::-1], strides=(0, 0, 0))
    b, c, out = Field("XVol", bx, ghost), Field("XVol", bx, ghost), Field("XVol", bx, ghost)
    m = Mask("XVol", np.zeros(1, dtype=np.uint32), gx, ghost)
    db = OpDB(n, n)
    i_sx, g_xs = db.interp("SVol", "XVol"), db.grad("XVol", "SVol")
    e = cond(m, 0.0, i_sx(g_xs(i_sx(a))) * exp(b) + sin(c))
    lim, _ = write_limits(out, e, True)
    return lim


def transport_run(phi0, u, v, w, lam, n, steps, dt, nu, threads=1):
    phi = np.ascontiguousarray(phi0, dtype=np.float64).copy()
    p1 = np.zeros_like(phi)
    pn = np.zeros_like(phi)
    lib().orc_transport_run(_p(phi), _p(p1), _p(pn), _p(u), _p(v), _p(w), _p(lam), int(n), int(steps),
                            ctypes.c_double(dt), ctypes.c_double(nu), int(threads))
    return phi


def heat_adjoint(T0, lam, gTN, n, steps, dt):
    """(dJ/dT0, dJ/dlam) for J with dJ/dT_N = gTN (windows; ghosts of the results are zero)."""
    gT = np.ascontiguousarray(gTN, dtype=np.float64).copy()
    glam = np.zeros_like(gT)
    lib().orc_heat_adjoint(_p(np.ascontiguousarray(T0)), _p(np.ascontiguousarray(lam)), _p(gT), _p(glam),
                           _i3(n), int(steps), ctypes.c_double(dt))
    return gT, glam


def reduce_field(f, g, op, interior=False):
    gz, gy, gx = f.shape
    lib().orc_reduce_field.restype = ctypes.c_double
    return lib().orc_reduce_field(_p(np.ascontiguousarray(f)), _i3((gx, gy, gz)), int(g), RED[op], int(interior))


def particle_ops(case, off=(0, 0, 0), nmax=None, fill=-7777.25):
    """CellToParticle(cell) and ParticleToCell(pval) of the oracle for one particle case (the dict
    of workloads.particle_inputs or a golden case).  The cell field's window starts at `off` and
    spans `nmax` (default: the whole allocation); allocation cells outside it keep `fill`."""
    glob = tuple(int(v) for v in case["glob"])
    nmax = glob if nmax is None else tuple(nmax)
    axes = int(case["axes"])
    cell = np.ascontiguousarray(case["cell"], dtype=np.float64)
    npart = len(case["psize"])
    pos = [np.ascontiguousarray(case[k], dtype=np.float64) for k in ("px", "py", "pz")]
    ptrs = [_p(pos[a]) if (axes >> a) & 1 else None for a in range(3)]
    psize = np.ascontiguousarray(case["psize"], dtype=np.float64)
    pval = np.ascontiguousarray(case["pval"], dtype=np.float64)
    d3 = (ctypes.c_double * 3)(*[float(v) for v in case["spacing"]])
    l3 = (ctypes.c_double * 3)(*[float(v) for v in case["low"]])
    c2p = np.empty(npart)
    p2c = np.full_like(cell, fill)
    L = lib()
    L.orc_cell_to_particle(d3, l3, _i3(case["ngm"]), _i3(glob), _i3(off), _i3(nmax), _p(cell), *ptrs, _p(psize),
                           ctypes.c_int64(npart), _p(c2p))
    L.orc_particle_to_cell(d3, l3, _i3(case["ngm"]), _i3(glob), _i3(off), _i3(nmax), _p(p2c), *ptrs, _p(psize),
                           ctypes.c_int64(npart), _p(pval))
    return c2p, p2c


def fill_periodic(f, g):
    gz, gy, gx = f.shape
    lib().orc_fill_periodic(_p(f), _i3((gx - 2 * g, gy - 2 * g, gz - 2 * g)), int(g))
    return f


def ghosts(expr, with_bc=True):
    """ghosts_with_bc() / ghosts_without_bc() of an expression (minus[3], plus[3])."""
    comp = _Compiled(expr)
    m = (ctypes.c_int32 * 3)()
    p = (ctypes.c_int32 * 3)()
    if lib().orc_ghosts(ctypes.byref(comp.e), int(with_bc), m, p) != 0:
        raise NeboError("ghost analysis failed")
    return tuple(m), tuple(p)
