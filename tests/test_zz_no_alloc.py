"""The allocation-free reduction entry point, called through the C ABI.

Some callers cannot allocate device memory where they reduce a field (a host framework that
reserved the GPU's memory up front in its own pool, or code running where the CUDA allocator
must not be entered).  nebo_reduce_noalloc serves them from a fixed device array.  This test
checks it against the allocating entry point nebo_reduce_async on the same fields, twice in a
row, so a second call that finds the first call's partials still in the array must still be
right.  It lives in its own file, collected last, and also passes when run alone.
"""
import ctypes

import numpy as np
import pytest

import spatialops_gb300 as N

pytestmark = pytest.mark.gpu

TOL = 1e-13  # relative, for the compensated sums; max/min are exact


def _fields():
    rng = np.random.default_rng(2024)
    a = rng.normal(size=(70, 66, 67))            # 65 x 64 x 68 interior, one ghost layer
    b = rng.uniform(-1.0, 1.0, size=(12, 9, 300))  # long rows, 2 ghost layers
    return [N.Field.from_numpy("SVol", a, 1), N.Field.from_numpy("SVol", b, 2, dtype="f32"),
            N.Field.from_numpy("SVol", a[:20, :20, :20].copy(), 1)]


def test_noalloc_reduction_matches_allocating_entry_point():
    import torch

    L = N.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ref = torch.zeros(1, dtype=torch.float64, device="cuda")
    got = torch.zeros(1, dtype=torch.float64, device="cuda")
    fields = _fields()
    for call in range(2):  # two calls in a row on every case
        for f in fields:
            d = f.desc()
            for op in ("sum", "max", "min", "norm"):
                for interior in (0, 1):
                    assert L.nebo_reduce_async(ctypes.byref(d), N.RED[op], interior,
                                               ctypes.c_void_p(ref.data_ptr()), stream) == 0
                    rc = L.nebo_reduce_noalloc(ctypes.byref(d), N.RED[op], interior,
                                               ctypes.c_void_p(got.data_ptr()), stream)
                    assert rc == 0, L.nebo_last_error()
                    torch.cuda.synchronize()
                    r, g = float(ref.item()), float(got.item())
                    if op in ("max", "min"):
                        assert g == r, (call, op, interior)
                    else:
                        assert abs(g - r) <= TOL * max(abs(r), 1e-300), (call, op, interior, g, r)
