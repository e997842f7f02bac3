"""Fused heat step on the GPU against the reference (golden vectors) and the oracle."""
import os

import numpy as np
import pytest

import oracle_dsl as O
import spatialops_gb300 as N
from spatialops_gb300 import workloads as W

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


def _run(lam, T0, steps, dt, dtype="f64", use_graph=True):
    T = N.Field.from_numpy("SVol", T0, 1, dtype=dtype)
    Tt = N.Field.from_numpy("SVol", np.zeros_like(T0), 1, dtype=dtype)
    L = N.Field.from_numpy("SVol", lam, 1, dtype=dtype)
    N.heat_run(T, Tt, L, steps, dt, use_graph=use_graph)
    return T


def test_heat_fp64_bitexact_vs_reference_golden():
    z = np.load(os.path.join(GOLD, "heat.npz"))
    T = _run(z["lam"], z["T0"], int(z["steps"]), float(z["dt"]))
    assert (_bits(T.numpy()) == _bits(z["f:T"])).all()
    # reductions: max exact; sum/norm within the compensated-sum bound
    assert N.nebo_max(T) == float(z["v:max"])
    absum = float(np.abs(z["f:T"]).sum())
    assert abs(N.nebo_sum(T) - float(z["v:sum"])) <= 1e-13 * absum
    assert abs(N.nebo_norm(T) - float(z["v:norm"])) <= 1e-13 * float(z["v:norm"])


@pytest.mark.parametrize("n,steps", [((64, 64, 64), 20), ((37, 29, 18), 7), ((33, 9, 65), 4), ((2, 8, 5), 3)])
def test_heat_fp64_bitexact_vs_oracle(n, steps):
    lam, T0, dt = W.heat_inputs(n, sigma=min(n) / 4.0)
    ref = O.heat_run(lam, T0, n, steps, dt)
    T = _run(lam, T0, steps, dt)
    assert (_bits(T.numpy()) == _bits(ref)).all()


# (40, 36, 20): the cp.async kernels; (48, 40, 20) in FP32: the bulk-copy kernel (rows in 8s)
@pytest.mark.parametrize("dtype,n", [("f64", (40, 36, 20)), ("f32", (40, 36, 20)), ("f32", (48, 40, 20))])
def test_heat_graph_equals_stream_launches(dtype, n):
    # the graph runs first: the FP32 kernels' per-device set-up must work inside the capture
    lam, T0, dt = W.heat_inputs(n, cfl=0.15)
    a = _run(lam, T0, 9, dt, use_graph=True, dtype=dtype).numpy()
    b = _run(lam, T0, 9, dt, use_graph=False, dtype=dtype).numpy()
    assert (a.view(np.uint8) == b.view(np.uint8)).all()


# bulk-copied row slabs (rows in 8s, even pitch: full width 256, narrower with a ragged last z
# chunk), 8-byte copies (odd row count), odd pitch
@pytest.mark.parametrize("n", [(64, 48, 40), (256, 256, 24), (200, 96, 37), (64, 44, 40), (37, 21, 19)])
def test_heat_fp32_error_vs_fp64_oracle(n):
    lam, T0, dt = W.heat_inputs(n, cfl=0.15)  # a stable step, so the error measure is meaningful
    ref = O.heat_run(lam, T0, n, 50, dt)
    T = _run(lam, T0, 50, dt, dtype="f32").numpy().astype(np.float64)
    err = np.abs(T - ref).max() / np.abs(ref).max()
    assert err <= 1e-5, err


def test_heat_general_spacing_bitexact():
    # non-unit spacing runs the reference's own operation order
    n = (20, 16, 12)
    lam, T0, _ = W.heat_inputs(n)
    sp = (1.5, 0.75, 2.0)
    dt = 0.1
    T = N.Field.from_numpy("SVol", T0, 1)
    Tt = N.Field.from_numpy("SVol", np.zeros_like(T0), 1)
    L = N.Field.from_numpy("SVol", lam, 1)
    N.heat_run(T, Tt, L, 3, dt, spacing=sp)
    # oracle: generic expression evaluator with the registered operators for L = n*spacing
    db = O.OpDB(n, tuple(n[i] * sp[i] for i in range(3)))
    cur = T0.copy()
    lamf = O.fill_periodic(lam.copy(), 1)
    for _ in range(3):
        O.fill_periodic(cur, 1)
        nxt = cur.copy()
        Tf, Lf, Nf = (O.Field("SVol", a, 1) for a in (cur, lamf, nxt))
        fx, fy, fz = O.FACES["SVol"]
        rhs = (db.div(fx, "SVol")(db.interp("SVol", fx)(Lf) * db.grad("SVol", fx)(Tf))
               + db.div(fy, "SVol")(db.interp("SVol", fy)(Lf) * db.grad("SVol", fy)(Tf))
               + db.div(fz, "SVol")(db.interp("SVol", fz)(Lf) * db.grad("SVol", fz)(Tf)))
        O.assign(Nf, Tf + dt * rhs)
        cur = nxt
    O.fill_periodic(cur, 1)
    assert (_bits(T.numpy()) == _bits(cur)).all()


def test_heat_rejects_in_place_and_bad_ghosts():
    T = N.Field("SVol", (8, 8, 8), 1)
    with pytest.raises(RuntimeError, match="in-place"):
        N.heat_step(T, T, T, 0.1)
    T2 = N.Field("SVol", (8, 8, 8), 2)
    with pytest.raises(RuntimeError, match="ghost"):
        N.heat_step(T2, N.Field("SVol", (8, 8, 8), 2), N.Field("SVol", (8, 8, 8), 2), 0.1)


# ---------------------------------------------------------------------------- fixed-point FP64 mode
def _run_ex(lam, T0, steps, dt, mode):
    T = N.Field.from_numpy("SVol", T0, 1)
    Tt = N.Field.from_numpy("SVol", np.zeros_like(T0), 1)
    L = N.Field.from_numpy("SVol", lam, 1)
    N.heat_run_ex(T, Tt, L, steps, dt, mode=mode)
    return T.numpy()


@pytest.mark.parametrize("n,steps", [((64, 64, 64), 100), ((37, 21, 19), 10), ((24, 20, 16), 50)])
def test_heat_fixed_point_vs_oracle(n, steps):
    """NEBO_HEAT_FIXED_POINT against the oracle's serial walk at the heat workload's own step
    (dt = 0.2 / max lambda, above the stability limit: the values grow, the scale follows them):
    within 1e-13 relative max-norm (test bound), ghost images included."""
    lam, T0, dt = W.heat_inputs(n, sigma=min(n) / 4.0)
    ref = O.heat_run(lam, T0, n, steps, dt)
    got = _run_ex(lam, T0, steps, dt, "fixed")
    err = float(np.abs(got - ref).max() / np.abs(ref).max())
    print(f"fixed-point heat {n} x {steps}: rel max-norm err {err:.2e}")
    assert err <= 1e-13, err


def test_heat_fixed_point_256_against_exact_kernel():
    n, steps = (256, 256, 256), 20
    lam, T0, dt = W.heat_inputs(n)
    a = _run_ex(lam, T0, steps, dt, "fixed")
    b = _run_ex(lam, T0, steps, dt, "exact")  # bit-identical to the oracle (tests above)
    err = float(np.abs(a - b).max() / np.abs(b).max())
    print(f"fixed-point heat 256^3 x {steps}: rel max-norm err vs the exact form {err:.2e}")
    assert err <= 1e-13, err


def test_heat_fixed_point_falls_back_to_fp64_on_non_finite_values():
    """A NaN in T: the fixed-point mode runs the exact FP64 form, bit for bit."""
    n, steps = (20, 16, 12), 4
    lam, T0, dt = W.heat_inputs(n)
    T0 = T0.copy()
    T0[5, 6, 7] = np.nan
    a = _run_ex(lam, T0, steps, dt, "fixed")
    b = _run_ex(lam, T0, steps, dt, "exact")
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


# ----------------------------------------------------------------- fixed-point state FP64 mode
@pytest.mark.parametrize("n,steps,cfl", [((64, 64, 64), 100, None), ((37, 21, 19), 10, None),
                                         ((24, 20, 16), 50, None), ((2, 8, 5), 3, None),
                                         ((24, 20, 16), 200, 0.1)])
def test_heat_fixed_state_vs_oracle(n, steps, cfl):
    """NEBO_HEAT_FIXED_STATE against the oracle's serial walk: the configuration's step (values
    grow x1.4 per step in the checkerboard mode, so the state is rescaled down) and a stable step
    (values decay, rescaled up); within 1e-13 relative max-norm, ghost images included."""
    kw = {} if cfl is None else {"cfl": cfl}
    lam, T0, dt = W.heat_inputs(n, sigma=min(n) / 4.0, **kw)
    ref = O.heat_run(lam, T0, n, steps, dt)
    got = _run_ex(lam, T0, steps, dt, "fixed_state")
    err = float(np.abs(got - ref).max() / np.abs(ref).max())
    print(f"fixed-state heat {n} x {steps}: rel max-norm err {err:.2e}")
    assert err <= 1e-13, err


def test_heat_fixed_state_256_against_exact_kernel():
    n, steps = (256, 256, 256), 20
    lam, T0, dt = W.heat_inputs(n)
    a = _run_ex(lam, T0, steps, dt, "fixed_state")
    b = _run_ex(lam, T0, steps, dt, "exact")
    err = float(np.abs(a - b).max() / np.abs(b).max())
    print(f"fixed-state heat 256^3 x {steps}: rel max-norm err vs the exact form {err:.2e}")
    assert err <= 1e-13, err


@pytest.mark.parametrize("where", ["T", "lam", "negative_lam"])
def test_heat_fixed_state_falls_back_to_fp64(where):
    """An infinity or a NaN in T or lambda, or a negative lambda (the integer form takes the lambda
    sums unsigned): the exact FP64 form runs on the integer buffers, bit for bit."""
    n, steps = (20, 16, 12), 5
    lam, T0, dt = W.heat_inputs(n)
    T0, lam = T0.copy(), lam.copy()
    if where == "T":
        T0[5, 6, 7] = np.nan
    elif where == "lam":
        lam[3, 4, 5] = np.inf
    else:
        lam[3, 4, 5] = -0.75
    a = _run_ex(lam, T0, steps, dt, "fixed_state")
    b = _run_ex(lam, T0, steps, dt, "exact")
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_heat_fixed_state_zero_steps_and_zero_field():
    n = (12, 10, 8)
    lam, T0, dt = W.heat_inputs(n)
    # zero steps: T keeps its values, ghosts filled (as the other modes)
    a = _run_ex(lam, T0, 0, dt, "fixed_state")
    b = _run_ex(lam, T0, 0, dt, "exact")
    assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    # an all-zero T stays zero
    z = _run_ex(lam, np.zeros_like(T0), 4, dt, "fixed_state")
    assert not z.any()


@pytest.mark.parametrize("mode", ["exact", "fixed", "fixed_state"])
def test_heat_run_ex_graph_equals_direct_launches(mode):
    """NEBO_HEAT_GRAPH: the captured call (conversions, steps, scratch from the stream-ordered pool)
    and its replay give the direct launches' bits."""
    n, steps = (24, 20, 16), 7
    lam, T0, dt = W.heat_inputs(n, cfl=0.15)

    def run(use_graph):
        T = N.Field.from_numpy("SVol", T0, 1)
        Tt = N.Field.from_numpy("SVol", np.zeros_like(T0), 1)
        L = N.Field.from_numpy("SVol", lam, 1)
        for _ in range(2):  # capture, then replay on the evolved state
            N.heat_run_ex(T, Tt, L, steps, dt, mode=mode, use_graph=use_graph)
        return T.numpy()

    assert np.array_equal(run(True).view(np.uint64), run(False).view(np.uint64))
