"""Scalar transport (FP64 and FP32-storage forms) and the heat adjoint on the GPU."""
import os

import numpy as np
import pytest

import oracle_dsl as O
import spatialops_gb300 as N
from spatialops_gb300 import workloads as W

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_transport_fp64_vs_reference_golden():
    z = np.load(os.path.join(GOLD, "transport.npz"))
    n = int(z["n"])
    t = N.Transport(z["phi0"], z["u"], z["v"], z["w"], z["lam"], n, float(z["dt"]), float(z["nu"]), dtype="f64")
    t.run(int(z["steps"]))
    assert _rel(t.phi.cpu().numpy(), z["f:phi"]) <= 1e-13


@pytest.mark.parametrize("n,steps", [(24, 6), (37, 3)])
def test_transport_fp64_vs_oracle(n, steps):
    phi, u, v, w, lam, dt, nu = W.transport_inputs(n)
    t = N.Transport(phi, u, v, w, lam, n, dt, nu, dtype="f64")
    t.run(steps)
    ref = O.transport_run(phi, u, v, w, lam, n, steps, dt, nu)
    assert _rel(t.phi.cpu().numpy(), ref) <= 1e-13


# even n: the packed cell-pair kernel (24 and 38 leave idle lanes in a tile); odd n: the generic one
@pytest.mark.parametrize("n,steps", [(32, 20), (24, 12), (38, 8), (21, 8)])
def test_transport_fp32_storage_error_vs_fp64_oracle(n, steps):
    phi, u, v, w, lam, dt, nu = W.transport_inputs(n)
    t = N.Transport(phi, u, v, w, lam, n, dt, nu, dtype="f32")
    t.run(steps)
    ref = O.transport_run(phi, u, v, w, lam, n, steps, dt, nu)
    assert _rel(t.phi.cpu().numpy(), ref) <= 1e-5


@pytest.mark.parametrize("n,steps", [(32, 6), (24, 4)])
def test_transport_fp32_tensor_staging_matches_cp_async_staging(n, steps):
    """n a multiple of 4 and lambda 16-byte aligned: the stage kernel stages phi and lambda as
    tensor tiles (24 also reads past the window's x end, where the tile is zero-filled); lambda
    8 bytes past a 16-byte boundary takes the cp.async form of the same kernel.  Same arithmetic
    on the same values, so the FP64 states are bit-identical."""
    import torch

    phi, u, v, w, lam, dt, nu = W.transport_inputs(n)
    a = N.Transport(phi, u, v, w, lam, n, dt, nu, dtype="f32")
    assert a.coef[3].data_ptr() % 16 == 0
    a.run(steps)
    b = N.Transport(phi, u, v, w, lam, n, dt, nu, dtype="f32")
    m = b.coef[3].numel()
    buf = torch.empty(m + 4, dtype=torch.float32, device="cuda")
    off = next(k for k in range(4) if (buf.data_ptr() + 4 * k) % 16 == 8)
    shifted = buf[off:off + m].view_as(b.coef[3])
    shifted.copy_(b.coef[3])
    b.coef[3] = shifted
    assert shifted.data_ptr() % 16 == 8
    b.run(steps)
    torch.cuda.synchronize()
    assert torch.equal(a.phi.view(torch.int64), b.phi.view(torch.int64))
    assert N.lib().nebo_stream_sync(None) == 0


def test_transport_velocity_is_divergence_free():
    n = 16
    _, u, v, w, _, _, _ = W.transport_inputs(n)
    g = 2
    i = slice(g, g + n)
    div = (u[i, i, g + 1:g + n + 1] - u[i, i, i]) + (v[i, g + 1:g + n + 1, i] - v[i, i, i]) + \
        (w[g + 1:g + n + 1, i, i] - w[i, i, i])
    assert np.abs(div).max() < 1e-12


# ---------------------------------------------------------------------------- adjoint
def _setup(n, steps, seed=8):
    lam, T0, dt, lam_t = W.adjoint_inputs(n, seed)
    Ttarget = O.heat_run(lam_t, T0, n, steps, dt)
    return lam, T0, dt, Ttarget


def _gpu_grad(lam, T0, Tt, steps, dt, every=0):
    F = lambda a: N.Field.from_numpy("SVol", a, 1)
    J, gT, gl = N.heat_gradient(F(T0), F(lam), F(Tt), steps, dt, every)
    return J, gT.numpy(), gl.numpy()


@pytest.mark.parametrize("every", [0, 1, 4, 50, N.CHECKPOINT_AUTO])
def test_adjoint_matches_oracle_adjoint(every):
    n, steps = (10, 9, 8), 13
    lam, T0, dt, Tt = _setup(n, steps)
    J, gT, gl = _gpu_grad(lam, T0, Tt, steps, dt, every)
    TN = O.heat_run(lam, T0, n, steps, dt)
    r = np.zeros_like(TN)
    r[1:-1, 1:-1, 1:-1] = (TN - Tt)[1:-1, 1:-1, 1:-1]
    ref_gT, ref_gl = O.heat_adjoint(T0, lam, r, n, steps, dt)
    I = (slice(1, -1),) * 3
    assert abs(J - 0.5 * float((r[I] ** 2).sum())) <= 1e-12 * max(J, 1e-300)
    assert _rel(gT[I], ref_gT[I]) <= 1e-12
    assert _rel(gl[I], ref_gl[I]) <= 1e-12


def test_adjoint_checkpointing_does_not_change_the_gradient():
    # sqrt(N) checkpoints (recomputed segments) and every state kept give the same bits
    n, steps = (12, 10, 9), 17
    lam, T0, dt, Tt = _setup(n, steps)
    J0, gT0, gl0 = _gpu_grad(lam, T0, Tt, steps, dt, 0)
    J1, gT1, gl1 = _gpu_grad(lam, T0, Tt, steps, dt, N.CHECKPOINT_AUTO)
    assert J0 == J1
    assert np.array_equal(gT0.view(np.uint64), gT1.view(np.uint64))
    assert np.array_equal(gl0.view(np.uint64), gl1.view(np.uint64))


def test_adjoint_dense_jacobian_8cubed():
    """dJ/dT0 = Jac^T r with the dense Jacobian of the (linear) map T0 -> T_N built column by column."""
    n, steps = (8, 8, 8), 10
    lam, T0, dt, Tt = _setup(n, steps)
    J, gT, _ = _gpu_grad(lam, T0, Tt, steps, dt)
    I = (slice(1, -1),) * 3
    TN = O.heat_run(lam, T0, n, steps, dt)
    r = (TN - Tt)[I].reshape(-1)
    jac = np.zeros((512, 512))
    for col in range(512):
        e = np.zeros_like(T0)
        e[I] = np.eye(1, 512, col).reshape(8, 8, 8)
        O.fill_periodic(e, 1)
        jac[:, col] = O.heat_run(lam, e, n, steps, dt)[I].reshape(-1)
    ref = jac.T @ r
    assert np.abs(gT[I].reshape(-1) - ref).max() <= 1e-11 * np.abs(ref).max()


@pytest.mark.parametrize("which", ["lam", "T0"])
def test_adjoint_vs_central_finite_differences(which):
    n, steps = (24, 20, 16), 40
    lam, T0, dt, Tt = _setup(n, steps)
    J, gT, gl = _gpu_grad(lam, T0, Tt, steps, dt)
    I = (slice(1, -1),) * 3
    rng = np.random.default_rng(9)
    F = lambda a: N.Field.from_numpy("SVol", a, 1)
    for _ in range(4):
        d = np.zeros_like(T0)
        d[I] = rng.normal(size=d[I].shape)
        O.fill_periodic(d, 1)
        eps = 1e-6
        if which == "lam":
            Jp = N.heat_gradient(F(T0), F(lam + eps * d), F(Tt), steps, dt)[0]
            Jm = N.heat_gradient(F(T0), F(lam - eps * d), F(Tt), steps, dt)[0]
            g = float((gl[I] * d[I]).sum())
        else:
            Jp = N.heat_gradient(F(T0 + eps * d), F(lam), F(Tt), steps, dt)[0]
            Jm = N.heat_gradient(F(T0 - eps * d), F(lam), F(Tt), steps, dt)[0]
            g = float((gT[I] * d[I]).sum())
        fd = (Jp - Jm) / (2 * eps)
        assert abs(fd - g) <= 1e-6 * abs(g), (fd, g)


def _periodic_direction(rng, like):
    d = np.zeros_like(like)
    I = (slice(1, -1),) * 3
    d[I] = rng.normal(size=d[I].shape)
    return O.fill_periodic(d, 1)


def test_adjoint_16_random_directions_autograd():
    """dJ/d(T0, lambda) through torch.autograd (HeatLoss) against FP64 central finite differences
    along 16 random joint directions (seed 9, eps = 1e-6)."""
    import torch

    from autograd_heat import HeatLoss

    n, steps = (24, 20, 16), 40
    lam, T0, dt, Tt = _setup(n, steps)
    cu = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    T0t = cu(T0).requires_grad_(True)
    lamt = cu(lam).requires_grad_(True)
    Ttt = cu(Tt)
    J = HeatLoss.apply(T0t, lamt, Ttt, steps, dt)
    J.backward()
    gT, gl = T0t.grad.cpu().numpy(), lamt.grad.cpu().numpy()
    rng = np.random.default_rng(9)
    eps = 1e-6
    for _ in range(16):
        dT, dl = _periodic_direction(rng, T0), _periodic_direction(rng, lam)
        Jp = float(HeatLoss.apply(cu(T0 + eps * dT), cu(lam + eps * dl), Ttt, steps, dt))
        Jm = float(HeatLoss.apply(cu(T0 - eps * dT), cu(lam - eps * dl), Ttt, steps, dt))
        fd = (Jp - Jm) / (2 * eps)
        g = float((gT * dT).sum() + (gl * dl).sum())
        assert abs(fd - g) <= 1e-6 * abs(g), (fd, g)


def test_adjoint_composes_with_autograd():
    """lambda = base * (1 + s * pert): dJ/ds by the chain rule through HeatLoss vs a central difference."""
    import torch

    from autograd_heat import HeatLoss

    n, steps = (16, 12, 10), 30
    lam, T0, dt, Tt = _setup(n, steps)
    cu = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    pert = cu(O.fill_periodic(np.random.default_rng(5).uniform(-1, 1, size=lam.shape), 1))
    base, T0t, Ttt = cu(lam), cu(T0), cu(Tt)
    s = torch.tensor(0.05, dtype=torch.float64, device="cuda", requires_grad=True)
    J = HeatLoss.apply(T0t, base * (1 + s * pert), Ttt, steps, dt)
    (dJds,) = torch.autograd.grad(J, s)
    eps = 1e-6
    Jp = float(HeatLoss.apply(T0t, base * (1 + (0.05 + eps) * pert), Ttt, steps, dt))
    Jm = float(HeatLoss.apply(T0t, base * (1 + (0.05 - eps) * pert), Ttt, steps, dt))
    fd = (Jp - Jm) / (2 * eps)
    assert abs(fd - float(dJds)) <= 1e-6 * abs(fd), (fd, float(dJds))


def test_adjoint_f32_face_products():
    """nebo_heat_gradient_ex(NEBO_PRODUCTS_F32): dJ/dT0 and J as the all-FP64 gradient (1e-12),
    dJ/dlambda within 1e-6 of the oracle adjoint, and against central differences."""
    n, steps = (24, 20, 16), 40
    lam, T0, dt, Tt = _setup(n, steps)
    F = lambda a: N.Field.from_numpy("SVol", a, 1)
    J, gT, gl = N.heat_gradient(F(T0), F(lam), F(Tt), steps, dt, products="f32")
    J64, gT64, gl64 = _gpu_grad(lam, T0, Tt, steps, dt)
    I = (slice(1, -1),) * 3
    gT, gl = gT.numpy(), gl.numpy()
    assert abs(J - J64) <= 1e-14 * J64
    assert _rel(gT[I], gT64[I]) <= 1e-12
    assert _rel(gl[I], gl64[I]) <= 1e-6
    rng = np.random.default_rng(9)
    eps = 1e-6
    for _ in range(4):
        dl = _periodic_direction(rng, lam)
        Jp = N.heat_gradient(F(T0), F(lam + eps * dl), F(Tt), steps, dt)[0]
        Jm = N.heat_gradient(F(T0), F(lam - eps * dl), F(Tt), steps, dt)[0]
        fd = (Jp - Jm) / (2 * eps)
        g = float((gl[I] * dl[I]).sum())
        assert abs(fd - g) <= 1e-6 * abs(g), (fd, g)
