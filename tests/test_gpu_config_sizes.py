"""Parity at the full sizes of the five workloads, where launch geometry differs from the small
cases (the chain's z split, the filter's one-wave flat runs, the transport pair kernel's tiles,
the patch work list).  Each test states the error it measures; tolerances are in the asserts.

* deep chain 256^3: out / filt within 1e-13 relative max-norm of the oracle; the fused max/min
  exactly those of the written filt and within 1e-13 of the oracle's; sum/norm within
  1e-13 * sum|x|; the written-cell set of `out` (pre-filled with a NaN payload)
  is exactly the reference's write region (calculate_actual_ghost, restated by the oracle);
* FP32 transport 512^3 + 2 ghosts, 50 RK2 steps: relative max-norm error against the FP64 GPU
  transport (which equals the oracle to 1e-13 on the small cases), and conservation of sum(phi);
* 512 patches x 200 steps: FP64 bit-exact against the oracle on the smallest, the largest and
  two random patches; FP32 and FP32x2 states: per-patch relative max error against FP64;
* adjoint 192^3 x 500 steps (sqrt(N) checkpoints): dJ/d(T0, lambda) against central finite
  differences along 16 random joint directions (eps = 1e-6), to 1e-6 relative; the FP32-forward
  gradient against the FP64 one (1e-4 relative max-norm).
"""
import os

import numpy as np
import pytest

import oracle_dsl as O
import spatialops_gb300 as N
from spatialops_gb300 import workloads as W

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1
NAN_SENTINEL = np.uint64(0x7FF4DEAD00C0FFEE)  # a NaN payload no computed value carries


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_deep_chain_256_vs_oracle_with_written_cells():
    import torch

    n = (256, 256, 256)
    a, b, c, pts = W.deep_inputs(n)
    bits = W.mask_bits_from_points(pts, n)
    o_out, o_filt = O.deep_run(a, b, c, bits, n, 1.0, THREADS)
    A = N.Field.from_numpy("SVol", a, 1)
    B = N.Field.from_numpy("XVol", b, 1)
    C = N.Field.from_numpy("XVol", c, 1)
    g = N.glob_dims("XVol", n, 1)
    # 1. written cells: out starts as the NaN payload everywhere
    sent = torch.full((g[2], g[1], g[0]), 0, dtype=torch.int64, device="cuda")
    sent.fill_(int(NAN_SENTINEL.astype(np.int64)))
    out = N.Field("XVol", n, 1, tensor=sent.view(torch.float64))
    filt = N.Field("XVol", n, 1)
    words = N.mask_from_points(N.mask_words(out.glob), out.glob, 1, pts)
    N.deep_chain(A, B, C, words, out, filt)
    unwritten = out.numpy().view(np.uint64) == NAN_SENTINEL
    lim = O.deep_write_region(n)
    want = np.ones(unwritten.shape, dtype=bool)
    want[lim[4] + 1:lim[5] + 1, lim[2] + 1:lim[3] + 1, lim[0] + 1:lim[1] + 1] = False
    assert np.array_equal(unwritten, want), f"written-cell set differs from the write region {lim}"
    o = out.numpy()
    w = ~want
    assert _rel(o[w], o_out[w]) <= 1e-13
    # 2. values and the fused reductions, out pre-filled with 0.0 as the oracle does
    out0, filt0 = N.Field("XVol", n, 1), N.Field("XVol", n, 1)
    red = torch.zeros(4, dtype=torch.float64, device="cuda")
    N.deep_chain(A, B, C, words, out0, filt0, reductions=red)
    f = filt0.numpy()
    err_out, err_filt = _rel(out0.numpy(), o_out), _rel(f, o_filt)
    print(f"deep 256^3: out rel err {err_out:.3e}, filt rel err {err_filt:.3e}")
    assert err_out <= 1e-13 and err_filt <= 1e-13
    r = red.cpu().numpy()
    mag = float(np.abs(o_filt).sum())
    # max/min: exactly those of the field the filter wrote (ghosts included), and within the
    # field's tolerance of the oracle's (the filter rounds 4 times where the reference rounds 27)
    assert r[1] == f.max() and r[2] == f.min()
    for k, op in ((1, "max"), (2, "min")):
        ref = O.reduce_field(o_filt, 1, op)
        assert abs(r[k] - ref) <= 1e-13 * float(np.abs(o_filt).max()), (op, r[k], ref)
    assert abs(r[0] - O.reduce_field(o_filt, 1, "sum")) <= 1e-13 * mag
    assert abs(r[3] - O.reduce_field(o_filt, 1, "norm")) <= 1e-13 * O.reduce_field(o_filt, 1, "norm")


def _transport(n, dtype, ins):
    import torch

    phi, u, v, w, lam, dt, nu = ins
    t = N.Transport.__new__(N.Transport)
    t.n, t.dt, t.nu = n, dt, nu
    t.dtype = N.F64 if dtype == "f64" else N.F32
    tdt = torch.float64 if dtype == "f64" else torch.float32
    t.phi = phi.clone()
    t.coef = [q.to(tdt).contiguous() for q in (u, v, w, lam)]
    t.work = torch.empty(N.lib().nebo_transport_work_bytes(int(n), t.dtype), dtype=torch.uint8, device="cuda")
    return t


def test_transport_fp32_512_cubed_50_steps_vs_fp64():
    import torch

    n, steps = 512, 50
    ins = W.transport_inputs_device(n)
    g = 2
    I = (slice(g, g + n),) * 3
    s0 = float(ins[0][I].sum())
    t64 = _transport(n, "f64", ins)
    t64.run(steps)
    torch.cuda.synchronize()
    p64 = t64.phi
    # conservation: the update is a divergence of face fluxes on a periodic grid
    s64 = float(p64[I].sum())
    mag = float(ins[0][I].abs().sum())
    assert abs(s64 - s0) <= 1e-12 * mag, (s64, s0)
    del t64
    t32 = _transport(n, "f32", ins)
    t32.run(steps)
    torch.cuda.synchronize()
    err = float((t32.phi[I] - p64[I]).abs().max() / p64[I].abs().max())
    s32 = float(t32.phi[I].sum())
    print(f"transport FP32 512^3 x {steps}: rel max-norm err vs FP64 {err:.3e}; "
          f"sum drift FP64 {abs(s64 - s0) / mag:.2e}, FP32 {abs(s32 - s0) / mag:.2e}")
    assert err <= 1e-5
    assert abs(s32 - s0) <= 1e-6 * mag


def _patchset(shapes, dtype, ins):
    import torch

    lam = np.array([t[0] for t in ins])
    dt = np.array([t[2] for t in ins])
    ps = N.PatchSet(shapes, lam, dt, dtype)
    ps.autotune()
    for p, (_, T0, _) in enumerate(ins):
        ps.window(0, p).copy_(torch.from_numpy(T0))
    ps.fill_ghosts(0)
    return ps


def test_patches_512_x_200_steps():
    steps = 200
    shapes = W.patch_shapes(512)
    ins = W.patch_inputs(shapes)
    ps64 = _patchset(shapes, "f64", ins)
    f64 = ps64.run(steps)
    ref = [ps64.window(f64, p).cpu().numpy() for p in range(len(shapes))]
    cells = np.prod(shapes.astype(np.int64), axis=1)
    rng = np.random.default_rng(1)
    check = sorted({int(np.argmin(cells)), int(np.argmax(cells)), *rng.choice(len(shapes), 2, replace=False).tolist()})
    for p in check:
        lam, T0, dt = ins[p]
        want = O.heat_run(np.full_like(T0, lam), T0, tuple(int(v) for v in shapes[p]), steps, dt, THREADS)
        assert np.array_equal(ref[p].view(np.uint64), want.view(np.uint64)), p
    del ps64
    for dtype, tol in (("f32", 1e-5), ("f32x2", 1e-6)):
        ps = _patchset(shapes, dtype, ins)
        fin = ps.run(steps)
        ps.sync(fin)
        errs = np.array([_rel(ps.window(fin, p).cpu().numpy(), ref[p]) for p in range(len(shapes))])
        print(f"patches {dtype} 512 x {steps} steps: per-patch rel max error max {errs.max():.3e}, "
              f"median {np.median(errs):.3e}")
        assert errs.max() <= tol
        del ps


def test_adjoint_192_cubed_500_steps_vs_finite_differences():
    import torch

    n, steps = (192, 192, 192), 500
    lam, T0, dt, lam_t = W.adjoint_inputs(n)
    F = lambda a: N.Field.from_numpy("SVol", a, 1)
    Tt, tmp = F(T0), N.Field("SVol", n, 1)
    N.heat_run(Tt, tmp, F(lam_t), steps, dt)
    torch.cuda.synchronize()
    J, gT, gl = N.heat_gradient(F(T0), F(lam), Tt, steps, dt)
    I = (slice(1, -1),) * 3
    gT, gl = gT.numpy(), gl.numpy()
    rng = np.random.default_rng(9)
    eps = 1e-6
    worst = 0.0
    for _ in range(16):
        dT = np.zeros_like(T0)
        dT[I] = rng.normal(size=dT[I].shape)
        O.fill_periodic(dT, 1)
        dl = np.zeros_like(lam)
        dl[I] = rng.normal(size=dl[I].shape)
        O.fill_periodic(dl, 1)
        Jp = N.heat_gradient(F(T0 + eps * dT), F(lam + eps * dl), Tt, steps, dt)[0]
        Jm = N.heat_gradient(F(T0 - eps * dT), F(lam - eps * dl), Tt, steps, dt)[0]
        fd = (Jp - Jm) / (2 * eps)
        g = float((gT[I] * dT[I]).sum() + (gl[I] * dl[I]).sum())
        worst = max(worst, abs(fd - g) / abs(g))
        assert abs(fd - g) <= 1e-6 * abs(g), (fd, g)
    print(f"adjoint 192^3 x {steps}: J {J:.6e}, worst FD relative difference over 16 directions {worst:.2e}")
    # the FP32-forward gradient (FP32 states and checkpoints, FP64 adjoint) against the FP64 one
    J32, gT32, gl32 = N.heat_gradient(F(T0), F(lam), Tt, steps, dt, forward="f32")
    e_T = float(np.abs(gT32.numpy()[I] - gT[I]).max() / np.abs(gT[I]).max())
    e_l = float(np.abs(gl32.numpy()[I] - gl[I]).max() / np.abs(gl[I]).max())
    print(f"adjoint 192^3 x {steps} FP32 forward: dJ/dT0 rel err {e_T:.2e}, dJ/dlambda rel err {e_l:.2e}, "
          f"J rel diff {abs(J32 - J) / J:.2e}")
    assert e_T <= 1e-4 and e_l <= 1e-4 and abs(J32 - J) <= 1e-4 * J
