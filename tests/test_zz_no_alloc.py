"""The allocation-free reduction entry point, called through the C ABI.

Some callers cannot allocate device memory where they reduce a field (a host framework that
reserved the GPU's memory up front in its own pool, or code running where the CUDA allocator
must not be entered).  nebo_reduce_noalloc serves them from a fixed device array.  The GPU test
checks it against the allocating entry point nebo_reduce_async on the same fields, twice in a
row, so a second call that finds the first call's partials still in the array must still be
right, and checks that the device's free memory does not move across the no-alloc calls.  It
lives in its own file, collected last, and also passes when run alone.  The CPU test checks the
size guard, which refuses a region before any CUDA call.
"""
import ctypes

import numpy as np
import pytest

import spatialops_gb300 as N

TOL = 1e-13  # relative, for the compensated sums; max/min are exact


def _fields():
    rng = np.random.default_rng(2024)
    a = rng.normal(size=(70, 66, 67))            # 65 x 64 x 68 interior, one ghost layer
    b = rng.uniform(-1.0, 1.0, size=(12, 9, 300))  # long rows, 2 ghost layers
    c = rng.normal(size=(260, 300, 6))           # 74 k rows: more rows than 4 blocks per SM
    return [N.Field.from_numpy("SVol", a, 1), N.Field.from_numpy("SVol", b, 2, dtype="f32"),
            N.Field.from_numpy("SVol", a[:20, :20, :20].copy(), 1), N.Field.from_numpy("SVol", c, 1)]


@pytest.mark.gpu
def test_noalloc_reduction_matches_allocating_entry_point():
    import torch

    L = N.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    ref = torch.zeros(1, dtype=torch.float64, device="cuda")
    got = torch.zeros(1, dtype=torch.float64, device="cuda")
    fields = _fields()
    wants = {}
    for f in fields:  # the allocating entry point's results, first
        d = f.desc()
        for op in ("sum", "max", "min", "norm"):
            for interior in (0, 1):
                assert L.nebo_reduce_async(ctypes.byref(d), N.RED[op], interior,
                                           ctypes.c_void_p(ref.data_ptr()), stream) == 0
                torch.cuda.synchronize()
                wants[(id(f), op, interior)] = float(ref.item())
    # one call loads the kernels (module loading may take device memory); then no call may move
    # the device's free memory
    d0 = fields[0].desc()
    assert L.nebo_reduce_noalloc(ctypes.byref(d0), 0, 0, ctypes.c_void_p(got.data_ptr()), stream) == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for call in range(2):  # two calls in a row on every case
        for f in fields:
            d = f.desc()
            for op in ("sum", "max", "min", "norm"):
                for interior in (0, 1):
                    rc = L.nebo_reduce_noalloc(ctypes.byref(d), N.RED[op], interior,
                                               ctypes.c_void_p(got.data_ptr()), stream)
                    assert rc == 0, L.nebo_last_error()
                    torch.cuda.synchronize()
                    r, g = wants[(id(f), op, interior)], float(got.item())
                    if op in ("max", "min"):
                        assert g == r, (call, op, interior)
                    else:
                        assert abs(g - r) <= TOL * max(abs(r), 1e-300), (call, op, interior, g, r)
    assert torch.cuda.mem_get_info()[0] == free0, "device free memory changed across no-alloc calls"


def test_noalloc_rejects_regions_beyond_its_row_limit_on_the_host():
    # 65536 x 65536 rows of one cell: more than 2^31 - 1 rows; refused before any CUDA call (the
    # data pointer is never touched)
    L = N.lib()
    d = N.NeboField()
    d.data = 0x1000
    d.glob[:] = (1, 65536, 65536)
    d.offset[:] = (0, 0, 0)
    d.extent[:] = (1, 65536, 65536)
    d.ghost_minus[:] = (0, 0, 0)
    d.ghost_plus[:] = (0, 0, 0)
    d.has_bc[:] = (0, 0, 0)
    d.bc_extra[:] = (0, 0, 0)
    d.dtype = N.F64
    rc = L.nebo_reduce_noalloc(ctypes.byref(d), 0, 0, ctypes.c_void_p(0x2000), None)
    assert rc == 1
    assert b"rows" in L.nebo_last_error()
