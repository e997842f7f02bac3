"""GB300-native Nebo field-expression evaluation: Python host mirror of the C-ABI library.

The product is libnebo_gb300.so (CUDA kernels for sm_103a behind the C ABI declared in
include/nebo_gb300.h) plus the drop-in C++ headers under include/spatialops.  This module binds
the C ABI with ctypes for tests and the benchmark.  It computes nothing itself: every call goes
to the CUDA library, and loading fails loudly if the library has not been built.

Names follow the reference's API (spatialops/NeboReductions.h, NeboStencilBuilder.h,
structured/SpatialField.h); errors raise RuntimeError with the library's "Nebo error in ..."
message, as the reference throws std::runtime_error.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_build", "libnebo_gb300.so")

F64, F32, F32X2 = 0, 1, 2
RED = {"sum": 0, "max": 1, "min": 2, "norm": 3}

# location type -> (offset, BCExtra), spatialops/structured/FVStaggeredLocationTypes.h:63-126
BCEXTRA = {
    "SVol": (0, 0, 0), "SSurfX": (1, 0, 0), "SSurfY": (0, 1, 0), "SSurfZ": (0, 0, 1),
    "XVol": (1, 0, 0), "XSurfX": (0, 0, 0), "XSurfY": (0, 1, 0), "XSurfZ": (0, 0, 1),
    "YVol": (0, 1, 0), "YSurfX": (1, 0, 0), "YSurfY": (0, 0, 0), "YSurfZ": (0, 0, 1),
    "ZVol": (0, 0, 1), "ZSurfX": (1, 0, 0), "ZSurfY": (0, 1, 0), "ZSurfZ": (0, 0, 0),
}


class NeboField(ctypes.Structure):
    """struct nebo_field (include/nebo_gb300.h)."""

    _fields_ = [
        ("data", ctypes.c_void_p),
        ("glob", ctypes.c_int32 * 3),
        ("offset", ctypes.c_int32 * 3),
        ("extent", ctypes.c_int32 * 3),
        ("ghost_minus", ctypes.c_int32 * 3),
        ("ghost_plus", ctypes.c_int32 * 3),
        ("has_bc", ctypes.c_int32 * 3),
        ("bc_extra", ctypes.c_int32 * 3),
        ("dtype", ctypes.c_int32),
    ]


class ParticleMesh(ctypes.Structure):
    """struct nebo_particle_mesh (include/nebo_gb300.h)."""

    _fields_ = [
        ("spacing", ctypes.c_double * 3),
        ("low", ctypes.c_double * 3),
        ("ghost_minus", ctypes.c_int32 * 3),
    ]


# (name, restype, argtypes) of every entry point declared in include/nebo_gb300.h
_P = ctypes.c_void_p
_FP = ctypes.POINTER(NeboField)
_I = ctypes.c_int
_D = ctypes.c_double
_I3 = ctypes.POINTER(ctypes.c_int32)
SIGNATURES = [
    ("nebo_status_string", ctypes.c_char_p, [_I]),
    ("nebo_last_error", ctypes.c_char_p, []),
    ("nebo_device_init", _I, [_I]),
    ("nebo_device_count", _I, [ctypes.POINTER(_I)]),
    ("nebo_alloc", _I, [ctypes.c_size_t, ctypes.POINTER(_P), _P]),
    ("nebo_free", _I, [_P, _P]),
    ("nebo_memcpy_h2d", _I, [_P, _P, ctypes.c_size_t, _P]),
    ("nebo_memcpy_d2h", _I, [_P, _P, ctypes.c_size_t, _P]),
    ("nebo_memcpy_d2d", _I, [_P, _P, ctypes.c_size_t, _P]),
    ("nebo_memset", _I, [_P, _I, ctypes.c_size_t, _P]),
    ("nebo_stream_sync", _I, [_P]),
    ("nebo_write_limits", _I, [_FP, _I, _I3, _I3, _I3]),
    ("nebo_fill_periodic", _I, [_FP, _P]),
    ("nebo_mask_from_points", _I, [_P, _I3, _I3, _P, ctypes.c_int32, _P]),
    ("nebo_reduce", _I, [_FP, _I, _I, ctypes.POINTER(_D), _P]),
    ("nebo_reduce_async", _I, [_FP, _I, _I, _P, _P]),
    ("nebo_reduce_noalloc", _I, [_FP, _I, _I, _P, _P]),
    ("nebo_reduce_all", _I, [_FP, _I, _P, _P]),
    ("nebo_heat_step", _I, [_FP, _FP, _FP, _D, ctypes.POINTER(_D), _P]),
    ("nebo_heat_run", _I, [_FP, _FP, _FP, _I, _D, ctypes.POINTER(_D), _I, _P]),
    ("nebo_deep_chain", _I, [_FP, _FP, _FP, _P, _FP, _FP, _D, _P]),
    ("nebo_deep_chain_reduce", _I, [_FP, _FP, _FP, _P, _FP, _FP, _D, _I, _P, _P]),
    ("nebo_patchset_create", _I, [ctypes.POINTER(_P), _I, _P, _P, _P, _I]),
    ("nebo_patchset_destroy", _I, [_P]),
    ("nebo_patchset_info", _I, [_P, _P, _P, _P, _P]),
    ("nebo_patchset_arena", _P, [_P, _I]),
    ("nebo_patchset_fill_ghosts", _I, [_P, _I, _P]),
    ("nebo_patchset_sync", _I, [_P, _I, _P]),
    ("nebo_patchset_autotune", _I, [_P, _P, _P]),
    ("nebo_patchset_run", _I, [_P, _I, _I, _I, ctypes.POINTER(_I), _P]),
    ("nebo_transport_work_bytes", ctypes.c_size_t, [_I, _I]),
    ("nebo_transport_run", _I, [_P, _P, _P, _P, _P, _I, _I, _D, _D, _I, _P, _P]),
    ("nebo_heat_adjoint_step", _I, [_FP, _FP, _FP, _FP, _FP, _D, _P]),
    ("nebo_heat_gradient", _I, [_FP, _FP, _FP, _I, _D, _I, _FP, _FP, ctypes.POINTER(_D), _P]),
    ("nebo_heat_gradient_ex", _I, [_FP, _FP, _FP, _I, _D, _I, _I, _FP, _FP, ctypes.POINTER(_D), _P]),
    ("nebo_fastmath_eval", _I, [_I, _P, _P, ctypes.c_size_t, _P]),
    ("nebo_box_filter", _I, [_FP, _FP, _I, _P, _P]),
    ("nebo_cell_to_particle", _I, [ctypes.POINTER(ParticleMesh), _P, _P, _P, _P, ctypes.c_int64, _FP, _P, _P]),
    ("nebo_particle_to_cell", _I, [ctypes.POINTER(ParticleMesh), _P, _P, _P, _P, ctypes.c_int64, _P, _FP, _P]),
    ("nebo_heat_run_ex", _I, [_FP, _FP, _FP, _I, _D, ctypes.POINTER(_D), _I, _P]),
    ("nebo_stencil_transpose", _I, [_FP, ctypes.POINTER(ctypes.c_int32), _FP, ctypes.c_int32, _P, _P, _I, _P]),
    ("nebo_kernel_launch_count", ctypes.c_ulonglong, []),
    ("nebo_profile_enable", _I, [_I]),
    ("nebo_profile_report", _I, [ctypes.c_char_p, ctypes.c_size_t, _I]),
]

_lib = None


def lib():
    """Load libnebo_gb300.so (raises if it was not built: there is no fallback path)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"Nebo error: CUDA library not built ({LIB_PATH}); run __graft_entry__.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc):
    if rc != 0:
        msg = lib().nebo_last_error().decode()
        raise RuntimeError(msg or lib().nebo_status_string(rc).decode())


def _i3(v):
    return (ctypes.c_int32 * 3)(*[int(t) for t in v])


def _stream(stream=None):
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def glob_dims(loc, n, ghost, bc=(0, 0, 0)):
    ex = BCEXTRA[loc]
    return tuple((n[i] + 2 * ghost + (ex[i] if bc[i] else 0)) if n[i] > 1 else 1 for i in range(3))


class Field:
    """A SpatialField-like handle: one device allocation (a torch tensor) + window/ghost/BC state.

    tensor has numpy shape (gz, gy, gx); the window covers the whole allocation.
    """

    def __init__(self, loc, n, ghost=1, bc=(0, 0, 0), dtype="f64", tensor=None, device="cuda"):
        import torch

        self.loc = loc
        self.n = tuple(int(v) for v in ((n,) * 3 if np.isscalar(n) else n))
        self.ghost = int(ghost)
        self.bc = tuple(int(b) for b in bc)
        self.dtype = F64 if dtype in ("f64", "float64", torch.float64) else F32
        g = glob_dims(loc, self.n, self.ghost, self.bc)
        self.glob = g
        tdt = torch.float64 if self.dtype == F64 else torch.float32
        if tensor is None:
            tensor = torch.zeros((g[2], g[1], g[0]), dtype=tdt, device=device)
        if tuple(tensor.shape) != (g[2], g[1], g[0]) or tensor.dtype != tdt or not tensor.is_contiguous():
            raise RuntimeError(f"Nebo error: tensor does not match the {loc} window {g[::-1]} ({tdt})")
        self.tensor = tensor

    @classmethod
    def from_numpy(cls, loc, arr, ghost=1, bc=(0, 0, 0), dtype="f64"):
        import torch

        gz, gy, gx = arr.shape
        ex = BCEXTRA[loc]
        n = tuple((d - 2 * ghost - (ex[i] if bc[i] else 0)) for i, d in enumerate((gx, gy, gz)))
        tdt = torch.float64 if dtype in ("f64", "float64") else torch.float32
        t = torch.from_numpy(np.ascontiguousarray(arr)).to(dtype=tdt, device="cuda")
        return cls(loc, n, ghost, bc, dtype, tensor=t)

    def desc(self):
        d = NeboField()
        d.data = self.tensor.data_ptr()
        d.glob[:] = self.glob
        d.offset[:] = (0, 0, 0)
        d.extent[:] = self.glob
        gm = [0 if self.glob[i] == 1 else self.ghost for i in range(3)]
        d.ghost_minus[:] = gm
        d.ghost_plus[:] = gm
        d.has_bc[:] = self.bc
        d.bc_extra[:] = [BCEXTRA[self.loc][i] if self.bc[i] else 0 for i in range(3)]
        d.dtype = self.dtype
        return d

    def numpy(self):
        return self.tensor.detach().cpu().numpy()


# ----------------------------------------------------------------------------- entry points
def device_count():
    n = ctypes.c_int(0)
    rc = lib().nebo_device_count(ctypes.byref(n))
    return n.value if rc == 0 else 0


def write_limits(lhs: Field, rhs_minus, rhs_plus, use_ghost=True):
    """calculate_actual_ghost + NeboField::assign limits, host code (no GPU needed)."""
    lim = (ctypes.c_int32 * 6)()
    d = lhs.desc() if isinstance(lhs, Field) else lhs
    _check(lib().nebo_write_limits(ctypes.byref(d), int(use_ghost), _i3(rhs_minus), _i3(rhs_plus), lim))
    return tuple(lim)


def fill_periodic(f: Field, stream=None):
    d = f.desc()
    _check(lib().nebo_fill_periodic(ctypes.byref(d), _stream(stream)))


def mask_words(glob):
    import torch

    nwords = (glob[0] * glob[1] * glob[2] + 31) // 32
    return torch.zeros(nwords, dtype=torch.int32, device="cuda")


def mask_from_points(words, glob, ghost, points, stream=None):
    """OR the bits of `points` (int32 (N,3), interior-relative) into device mask words."""
    import torch

    pts = torch.as_tensor(np.ascontiguousarray(points, dtype=np.int32)).to("cuda")
    _check(lib().nebo_mask_from_points(ctypes.c_void_p(words.data_ptr()), _i3(glob), _i3((ghost,) * 3),
                                       ctypes.c_void_p(pts.data_ptr()), len(points), _stream(stream)))
    return words


def _reduce(f, op, interior, stream=None):
    out = ctypes.c_double()
    d = f.desc()
    _check(lib().nebo_reduce(ctypes.byref(d), RED[op], int(interior), ctypes.byref(out), _stream(stream)))
    return out.value


def nebo_sum(f, stream=None): return _reduce(f, "sum", False, stream)
def nebo_max(f, stream=None): return _reduce(f, "max", False, stream)
def nebo_min(f, stream=None): return _reduce(f, "min", False, stream)
def nebo_norm(f, stream=None): return _reduce(f, "norm", False, stream)
def nebo_sum_interior(f, stream=None): return _reduce(f, "sum", True, stream)
def nebo_max_interior(f, stream=None): return _reduce(f, "max", True, stream)
def nebo_min_interior(f, stream=None): return _reduce(f, "min", True, stream)
def nebo_norm_interior(f, stream=None): return _reduce(f, "norm", True, stream)


def reduce_async(f, op, interior, d_result, stream=None):
    d = f.desc()
    _check(lib().nebo_reduce_async(ctypes.byref(d), RED[op], int(interior), ctypes.c_void_p(d_result.data_ptr()),
                                   _stream(stream)))


def reduce_all(f, interior, d_out4, stream=None):
    """sum, max, min, norm of one field in a single pass into a device float64 tensor of 4."""
    d = f.desc()
    _check(lib().nebo_reduce_all(ctypes.byref(d), int(interior), ctypes.c_void_p(d_out4.data_ptr()), _stream(stream)))


def heat_step(T, Tout, lam, dt, spacing=(1.0, 1.0, 1.0), stream=None):
    a, b, c = T.desc(), Tout.desc(), lam.desc()
    sp = (ctypes.c_double * 3)(*spacing)
    _check(lib().nebo_heat_step(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), float(dt), sp, _stream(stream)))


def heat_run(T, Ttmp, lam, steps, dt, spacing=(1.0, 1.0, 1.0), use_graph=True, stream=None):
    a, b, c = T.desc(), Ttmp.desc(), lam.desc()
    sp = (ctypes.c_double * 3)(*spacing)
    _check(lib().nebo_heat_run(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), int(steps), float(dt), sp,
                               int(use_graph), _stream(stream)))


HEAT_MODES = {"exact": 0, "fixed": 1, "fixed_state": 2}  # NEBO_HEAT_EXACT, _FIXED_POINT, _FIXED_STATE
HEAT_GRAPH = 0x100  # NEBO_HEAT_GRAPH


def heat_run_ex(T, Ttmp, lam, steps, dt, mode="fixed", spacing=(1.0, 1.0, 1.0), stream=None, use_graph=False):
    """nebo_heat_run_ex: `steps` FP64 Euler steps, the result in T; mode "fixed" computes the fluxes
    on the integer pipe, "fixed_state" keeps the whole run's state in 64-bit integers (both within
    a few 2^-60 of max|T| per step of the exact form); use_graph captures the call in a CUDA graph
    once and replays it for the same arguments."""
    a, b, c = T.desc(), Ttmp.desc(), lam.desc()
    sp = (ctypes.c_double * 3)(*spacing)
    _check(lib().nebo_heat_run_ex(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), int(steps), float(dt), sp,
                                  HEAT_MODES[mode] | (HEAT_GRAPH if use_graph else 0), _stream(stream)))


def deep_chain(a, b, c, words, out, filt, dx=1.0, stream=None, reductions=None, interior=False):
    """out <<= cond(mask,0)(Interp(Grad(Interp(a)))*exp(b)+sin(c)); filt <<= BoxFilter(out).

    reductions: optional float64 CUDA tensor of 4 that receives {sum, max, min, norm} of filt
    (valid ghosts included unless interior), folded into the filter kernel."""
    da, db, dc, do, df = a.desc(), b.desc(), c.desc(), out.desc(), filt.desc()
    if reductions is None:
        _check(lib().nebo_deep_chain(ctypes.byref(da), ctypes.byref(db), ctypes.byref(dc),
                                     ctypes.c_void_p(words.data_ptr()), ctypes.byref(do), ctypes.byref(df), float(dx),
                                     _stream(stream)))
        return
    _check(lib().nebo_deep_chain_reduce(ctypes.byref(da), ctypes.byref(db), ctypes.byref(dc),
                                        ctypes.c_void_p(words.data_ptr()), ctypes.byref(do), ctypes.byref(df),
                                        float(dx), int(interior), ctypes.c_void_p(reductions.data_ptr()),
                                        _stream(stream)))


def box_filter(src, dst, reductions=None, interior=False, stream=None):
    """dst <<= BoxFilter3D(src) (27 points x 1/27) on the interior; with `reductions` (a float64
    device tensor of 4) also {sum, max, min, norm} of dst in the same pass."""
    a, b = src.desc(), dst.desc()
    rp = ctypes.c_void_p(reductions.data_ptr()) if reductions is not None else None
    _check(lib().nebo_box_filter(ctypes.byref(a), ctypes.byref(b), int(bool(interior)), rp, _stream(stream)))
    return dst


def kernel_launch_count():
    return int(lib().nebo_kernel_launch_count())


def profile_enable(on=True):
    _check(lib().nebo_profile_enable(int(on)))


def profile_report(reset=True):
    """{kernel: {"launches": n, "ms": total}} for launches timed since the last reset."""
    import json

    buf = ctypes.create_string_buffer(1 << 16)
    _check(lib().nebo_profile_report(buf, len(buf), int(reset)))
    return json.loads(buf.value.decode())


class PatchSet:
    """Batched periodic heat patches (nebo_patchset_*): one persistent launch per step."""

    def __init__(self, shapes, lam, dt, dtype="f64"):
        self.shapes = np.ascontiguousarray(shapes, dtype=np.int32).reshape(-1, 3)
        self.npatch = len(self.shapes)
        self.lam = np.ascontiguousarray(lam, dtype=np.float64)
        self.dt = np.ascontiguousarray(dt, dtype=np.float64)
        self.dtype = {"f64": F64, "f32": F32, "f32x2": F32X2}[dtype]
        self.esize = 8  # the visible arenas hold FP64 states in every mode
        h = ctypes.c_void_p()
        _check(lib().nebo_patchset_create(ctypes.byref(h), self.npatch, ctypes.c_void_p(self.shapes.ctypes.data),
                                          ctypes.c_void_p(self.lam.ctypes.data), ctypes.c_void_p(self.dt.ctypes.data),
                                          self.dtype))
        self.h = h
        self._info()

    def _info(self):
        total = ctypes.c_int64()
        self.offsets = np.zeros(self.npatch, dtype=np.int64)
        self.log2tx = np.zeros(self.npatch, dtype=np.int32)
        nitems = ctypes.c_int32()
        _check(lib().nebo_patchset_info(self.h, ctypes.byref(total), ctypes.c_void_p(self.offsets.ctypes.data),
                                        ctypes.c_void_p(self.log2tx.ctypes.data), ctypes.byref(nitems)))
        self.total, self.nitems = total.value, nitems.value

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().nebo_patchset_destroy(self.h)
        except Exception:
            pass

    def arena(self, which):
        """The arena as a torch tensor view (no copy)."""
        import torch

        ptr = lib().nebo_patchset_arena(self.h, int(which))
        nbytes = self.total * self.esize
        cls = ctypes.c_double if self.dtype == F64 else ctypes.c_float
        # wrap the raw device pointer through a CUDA array interface
        class _CAI:
            pass
        obj = _CAI()
        obj.__cuda_array_interface__ = {"shape": (self.total,), "typestr": "<f8",
                                        "data": (ptr, False), "version": 3, "strides": None}
        del cls, nbytes
        return torch.as_tensor(obj, device="cuda")

    def window(self, which, p):
        nx, ny, nz = (int(v) for v in self.shapes[p])
        n = (nx + 2) * (ny + 2) * (nz + 2)
        o = int(self.offsets[p])
        return self.arena(which)[o:o + n].view(nz + 2, ny + 2, nx + 2)

    def fill_ghosts(self, which=0, stream=None):
        _check(lib().nebo_patchset_fill_ghosts(self.h, int(which), _stream(stream)))

    def autotune(self, stream=None):
        out = np.zeros(self.npatch, dtype=np.int32)
        _check(lib().nebo_patchset_autotune(self.h, _stream(stream), ctypes.c_void_p(out.ctypes.data)))
        self._info()
        return out

    def run(self, steps, start=0, use_graph=True, stream=None):
        fin = ctypes.c_int()
        _check(lib().nebo_patchset_run(self.h, int(start), int(steps), int(use_graph), ctypes.byref(fin),
                                       _stream(stream)))
        return fin.value

    def sync(self, which, stream=None):
        """Make FP64 arena `which` hold the state (needed after run in the two-float mode)."""
        _check(lib().nebo_patchset_sync(self.h, int(which), _stream(stream)))


class Transport:
    """Scalar transport state on the GPU (nebo_transport_run): phi FP64, coefficients in dtype."""

    def __init__(self, phi0, u, v, w, lam, n, dt, nu, dtype="f32"):
        import torch

        self.n, self.dt, self.nu = n, dt, nu
        self.dtype = F64 if dtype == "f64" else F32
        tdt = torch.float64 if self.dtype == F64 else torch.float32
        self.phi = torch.from_numpy(np.ascontiguousarray(phi0)).to(device="cuda", dtype=torch.float64)
        self.coef = [torch.from_numpy(np.ascontiguousarray(a)).to(device="cuda", dtype=tdt) for a in (u, v, w, lam)]
        nb = lib().nebo_transport_work_bytes(int(n), self.dtype)
        self.work = torch.empty(nb, dtype=torch.uint8, device="cuda")

    def run(self, steps, stream=None):
        c = [ctypes.c_void_p(t.data_ptr()) for t in self.coef]
        _check(lib().nebo_transport_run(ctypes.c_void_p(self.phi.data_ptr()), c[0], c[1], c[2], c[3], int(self.n),
                                        int(steps), float(self.dt), float(self.nu), self.dtype,
                                        ctypes.c_void_p(self.work.data_ptr()), _stream(stream)))


CHECKPOINT_AUTO = -1  # NEBO_CHECKPOINT_AUTO: keep every state when they fit in device memory


FORWARD_F32 = 2  # NEBO_FORWARD_F32


def heat_gradient(T0, lam, Ttarget, steps, dt, checkpoint_every=0, stream=None, products="f64", forward="f64"):
    """(J, dJ/dT0, dJ/dlambda) for J = 1/2 sum (T_N - T_target)^2 (fields: SVol, 1 ghost, FP64).

    checkpoint_every: 0 = ceil(sqrt(steps)); CHECKPOINT_AUTO = every state when they fit.
    products="f32": the lambda gradient's face products in FP32 (nebo_heat_gradient_ex).
    forward="f32": the forward states (and checkpoints) in FP32, the adjoint in FP64."""
    gT = Field(T0.loc, T0.n, T0.ghost)
    gl = Field(T0.loc, T0.n, T0.ghost)
    J = ctypes.c_double()
    a, b, c, d, e = T0.desc(), lam.desc(), Ttarget.desc(), gT.desc(), gl.desc()
    if products == "f64" and forward == "f64":
        _check(lib().nebo_heat_gradient(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), int(steps), float(dt),
                                        int(checkpoint_every), ctypes.byref(d), ctypes.byref(e), ctypes.byref(J),
                                        _stream(stream)))
    else:
        _check(lib().nebo_heat_gradient_ex(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), int(steps),
                                           float(dt), int(checkpoint_every),
                                           {"f64": 0, "f32": 1}[products] | (FORWARD_F32 if forward == "f32" else 0),
                                           ctypes.byref(d),
                                           ctypes.byref(e), ctypes.byref(J), _stream(stream)))
    return J.value, gT, gl


def stencil_transpose(dst_bar, limits, src_bar, points, coefs, accumulate=False, stream=None):
    """src_bar(j) (+)= sum_k coefs[k] * dst_bar(j - points[k]) over j - points[k] in limits: the
    transpose of dst(i) = sum_k coefs[k] * src(i + points[k]) on the write region `limits`."""
    pts = np.ascontiguousarray(points, dtype=np.int32).reshape(-1, 3)
    cf = np.ascontiguousarray(coefs, dtype=np.float64).reshape(-1)
    if len(pts) != len(cf):
        raise RuntimeError("Nebo error in stencil_transpose: one coefficient per point")
    lim = (ctypes.c_int32 * 6)(*[int(v) for v in limits])
    a, b = dst_bar.desc(), src_bar.desc()
    _check(lib().nebo_stencil_transpose(ctypes.byref(a), lim, ctypes.byref(b), len(pts),
                                        ctypes.c_void_p(pts.ctypes.data), ctypes.c_void_p(cf.ctypes.data),
                                        int(bool(accumulate)), _stream(stream)))


def heat_adjoint_step(Tk, Ain, Aout, lam, glam, dt, stream=None):
    a, b, c, d, e = Tk.desc(), Ain.desc(), Aout.desc(), lam.desc(), glam.desc()
    _check(lib().nebo_heat_adjoint_step(ctypes.byref(a), ctypes.byref(b), ctypes.byref(c), ctypes.byref(d),
                                        ctypes.byref(e), float(dt), _stream(stream)))


def fastmath_eval(fn, x, stream=None):
    """Element-wise table-driven FP64 exp ("exp") or sin ("sin") of a CUDA float64 tensor."""
    import torch

    y = torch.empty_like(x)
    _check(lib().nebo_fastmath_eval({"exp": 0, "sin": 1}[fn], ctypes.c_void_p(x.data_ptr()),
                                    ctypes.c_void_p(y.data_ptr()), x.numel(), _stream(stream)))
    return y


# ----------------------------------------------------------------------------- particles
def _particle_args(cell, px, py, pz, psize, spacing, low, ghost_minus):
    d = cell.desc() if isinstance(cell, Field) else cell
    m = ParticleMesh()
    m.spacing[:] = [float(v) for v in spacing]
    m.low[:] = [float(v) for v in low]
    m.ghost_minus[:] = list(d.ghost_minus) if ghost_minus is None else [int(v) for v in ghost_minus]
    ptr = [ctypes.c_void_p(t.data_ptr()) if t is not None else None for t in (px, py, pz, psize)]
    n = int(psize.numel()) if psize is not None else 0
    return d, m, ptr, n


def cell_to_particle(cell, px, py, pz, psize, dest, spacing, low, ghost_minus=None, stream=None):
    """Particle::CellToParticle::apply_to_field (spatialops/particles/ParticleOperators.h:313-398):
    dest[p] = the particle-volume-weighted sum of the cell values its box covers.  cell is a Field
    (or a NeboField descriptor); px, py, pz (None = axis off), psize and dest are float64 device
    tensors of one value per particle; spacing / low are the operator's state after its
    constructor; ghost_minus defaults to the field's ghost cells on the - faces."""
    d, m, ptr, n = _particle_args(cell, px, py, pz, psize, spacing, low, ghost_minus)
    _check(lib().nebo_cell_to_particle(ctypes.byref(m), *ptr, ctypes.c_int64(n), ctypes.byref(d),
                                       ctypes.c_void_p(dest.data_ptr()), _stream(stream)))
    return dest


def particle_to_cell(src, px, py, pz, psize, cell, spacing, low, ghost_minus=None, stream=None):
    """Particle::ParticleToCell::apply_to_field (spatialops/particles/ParticleOperators.h:186-273):
    every window cell of `cell` = the sum, in particle order, of src[p] x the fraction of particle
    p's volume inside it (0 where no particle reaches).  Synchronises the stream once."""
    d, m, ptr, n = _particle_args(cell, px, py, pz, psize, spacing, low, ghost_minus)
    _check(lib().nebo_particle_to_cell(ctypes.byref(m), *ptr, ctypes.c_int64(n),
                                       ctypes.c_void_p(src.data_ptr()) if src is not None else None,
                                       ctypes.byref(d), _stream(stream)))
    return cell
