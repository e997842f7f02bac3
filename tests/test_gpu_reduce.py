"""Reductions and periodic ghost fill on the GPU."""
import numpy as np
import pytest

import oracle_dsl as O
import spatialops_gb300 as N

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape,ghost", [((10, 9, 8), 1), ((66, 66, 66), 1), ((7, 300, 5), 2), ((130, 3, 4), 1)])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_reductions_vs_oracle(shape, ghost, dtype):
    rng = np.random.default_rng(sum(shape))
    g = tuple(s + 2 * ghost for s in shape)
    a = rng.normal(size=(g[2], g[1], g[0]))
    if dtype == "f32":
        a = a.astype(np.float32).astype(np.float64)
    f = N.Field.from_numpy("SVol", a, ghost, dtype=dtype)
    for interior in (False, True):
        for op in ("sum", "max", "min", "norm"):
            ref = O.reduce_field(a, ghost, op, interior)
            got = N._reduce(f, op, interior)
            if op in ("max", "min"):
                assert got == ref
            else:
                scale = float(np.abs(a).sum()) if op == "sum" else abs(ref)
                assert abs(got - ref) <= 1e-13 * scale, (op, got, ref)


@pytest.mark.parametrize("n,g", [((9, 7, 5), 1), ((12, 12, 12), 2), ((2, 6, 4), 1)])
def test_fill_periodic_vs_oracle(n, g):
    rng = np.random.default_rng(3)
    a = rng.normal(size=(n[2] + 2 * g, n[1] + 2 * g, n[0] + 2 * g))
    f = N.Field.from_numpy("SVol", a, g)
    N.fill_periodic(f)
    ref = O.fill_periodic(a.copy(), g)
    assert (f.numpy() == ref).all()


@pytest.mark.parametrize("shape,ghost", [((10, 9, 8), 1), ((66, 66, 66), 1), ((7, 300, 5), 2)])
@pytest.mark.parametrize("dtype", ["f64", "f32"])
def test_reduce_all_single_pass_vs_oracle(shape, ghost, dtype):
    import torch

    rng = np.random.default_rng(7 + sum(shape))
    g = tuple(s + 2 * ghost for s in shape)
    a = rng.normal(size=(g[2], g[1], g[0]))
    if dtype == "f32":
        a = a.astype(np.float32).astype(np.float64)
    f = N.Field.from_numpy("SVol", a, ghost, dtype=dtype)
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    for interior in (False, True):
        N.reduce_all(f, interior, out)
        s, mx, mn, nrm = out.cpu().numpy()
        assert mx == O.reduce_field(a, ghost, "max", interior)
        assert mn == O.reduce_field(a, ghost, "min", interior)
        ref_s = O.reduce_field(a, ghost, "sum", interior)
        assert abs(s - ref_s) <= 1e-13 * float(np.abs(a).sum())
        ref_n = O.reduce_field(a, ghost, "norm", interior)
        assert abs(nrm - ref_n) <= 1e-13 * ref_n
