"""Batched patches (one persistent launch per step over a device patch table) vs the oracle."""
import numpy as np
import pytest

import oracle_dsl as O
import spatialops_gb300 as N
from spatialops_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _setup(shapes, dtype, autotune):
    ins = W.patch_inputs(shapes)
    lam = np.array([t[0] for t in ins])
    dt = np.array([t[2] for t in ins])
    ps = N.PatchSet(shapes, lam, dt, dtype)
    chosen = ps.autotune() if autotune else None
    import torch

    for p, (_, T0, _) in enumerate(ins):
        ps.window(0, p).copy_(torch.from_numpy(T0))
    ps.fill_ghosts(0)
    return ps, ins, chosen


def _oracle(shape, lam, T0, dt, steps):
    L = np.full_like(T0, lam)
    return O.heat_run(L, T0, tuple(int(v) for v in shape), steps, dt)


@pytest.mark.parametrize("use_graph", [True, False])
def test_patches_fp64_bitexact(use_graph):
    rng = np.random.default_rng(11)
    shapes = rng.integers(2, 24, size=(14, 3)).astype(np.int32)
    shapes[0] = (2, 2, 2)
    shapes[1] = (17, 3, 33)
    ps, ins, _ = _setup(shapes, "f64", autotune=False)
    fin = ps.run(7, use_graph=use_graph)
    for p in range(len(shapes)):
        ref = _oracle(shapes[p], ins[p][0], ins[p][1], ins[p][2], 7)
        got = ps.window(fin, p).cpu().numpy()
        assert (got.view(np.uint64) == ref.view(np.uint64)).all(), p


def test_patches_autotune_keeps_results():
    shapes = np.array([[16, 20, 9], [40, 12, 18], [70, 9, 11], [33, 33, 8], [96, 17, 5]], dtype=np.int32)
    ps, ins, chosen = _setup(shapes, "f64", autotune=True)
    assert set(chosen.tolist()) <= {4, 5, 6}
    fin = ps.run(5)
    for p in range(len(shapes)):
        ref = _oracle(shapes[p], ins[p][0], ins[p][1], ins[p][2], 5)
        assert (ps.window(fin, p).cpu().numpy().view(np.uint64) == ref.view(np.uint64)).all(), p


@pytest.mark.parametrize("dtype,steps,tol", [
    ("f32", 200, 1e-5),     # FP32 storage and arithmetic: the batched FP32 form (half the bytes)
    ("f32x2", 200, 1e-6),   # two-float state, FP32 arithmetic only
])
def test_patches_fp32_error_vs_fp64_oracle(dtype, steps, tol):
    rng = np.random.default_rng(5)
    shapes = rng.integers(8, 40, size=(10, 3)).astype(np.int32)
    ps, ins, _ = _setup(shapes, dtype, autotune=True)
    fin = ps.run(steps)
    ps.sync(fin)
    for p in range(len(shapes)):
        ref = _oracle(shapes[p], ins[p][0], ins[p][1], ins[p][2], steps)
        got = ps.window(fin, p).cpu().numpy()
        err = np.abs(got - ref).max() / np.abs(ref).max()
        print(f"patch {p} {tuple(shapes[p])} {dtype} {steps} steps: relative max error {err:.3e}")
        assert err <= tol, (p, err)
