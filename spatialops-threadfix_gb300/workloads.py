"""Seeded synthetic inputs for the five Nebo workloads (no dataset is involved).

Every array is a full ghosted window in the reference's memory layout: x fastest, shape
(gz, gy, gx) in numpy order, glob = n + 2*ghosts per axis (no boundary-condition cells).
numpy's PCG64 generator is platform independent, so the same seed gives the same inputs on
the x86 build host and on the Arm GPU host.

Workloads (sizes are the full-scale ones; tests pass smaller n):
  heat       SVol n^3 + 1 ghost, lambda ~ U[0.5,1.5] (seed 1), T0 = Gaussian bump
             (sigma 8 cells, amplitude 1) + N(0, 1e-3) noise (seed 2), dt = 0.2/max(lambda).
             That dt is the workload's stated one; it is above the 3-D forward-Euler limit
             dt*lambda <= 1/6, so the noise's checkerboard mode grows by |1 - 12*0.2| = 1.4 per
             step.  Bitwise parity does not care; error measurements use cfl = 0.15 instead.
  deep       a (SVol), b, c (XVol) ~ U(-1,1) (seeds 3,4,5), mask = 5% of cells (seed 6) plus
             every interior cell with an index in {0, n-1}
  patches    edge lengths ~ U{16..96} per axis (seed 7), per-patch scalar lambda, Gaussian T0,
             dt = 0.15/lambda (stable; the workload does not state dt)
  adjoint    heat inputs with dt = 0.15/max(lambda) (stable; not stated by the workload);
             target from lambda*(1 + 0.1 sin(2 pi x/L)) (seed 8)
  transport  SVol n^3 + 2 ghosts; u,v,w discretely divergence-free (curl of a 4-mode vector
             potential, seed 10), |u| <= 1; lambda ~ U(0.5,1.5)
"""
from __future__ import annotations

import numpy as np


def window_shape(n, g):
    n = (n, n, n) if np.isscalar(n) else tuple(n)
    return (n[2] + 2 * g, n[1] + 2 * g, n[0] + 2 * g)


def fill_periodic(a, g):
    """Periodic ghost fill of a (gz, gy, gx) array in place: ghosts take wrapped interior values."""
    gz, gy, gx = a.shape
    n = (gx - 2 * g, gy - 2 * g, gz - 2 * g)
    ix = (np.arange(-g, n[0] + g) % n[0]) + g
    iy = (np.arange(-g, n[1] + g) % n[1]) + g
    iz = (np.arange(-g, n[2] + g) % n[2]) + g
    a[...] = a[np.ix_(iz, iy, ix)]
    return a


def gaussian_bump(n, g, sigma=8.0, amp=1.0):
    n = (n, n, n) if np.isscalar(n) else tuple(n)
    zz, yy, xx = np.meshgrid(
        np.arange(-g, n[2] + g) + 0.5 - n[2] / 2.0,
        np.arange(-g, n[1] + g) + 0.5 - n[1] / 2.0,
        np.arange(-g, n[0] + g) + 0.5 - n[0] / 2.0,
        indexing="ij",
    )
    return amp * np.exp(-(xx * xx + yy * yy + zz * zz) / (2.0 * sigma * sigma))


def heat_inputs(n, seed_lam=1, seed_t=2, sigma=8.0, cfl=0.2):
    """lambda, T0 (both full windows, ghosts filled periodically) and dt = cfl/max(lambda)."""
    shp = window_shape(n, 1)
    lam = np.random.default_rng(seed_lam).uniform(0.5, 1.5, size=shp)
    T0 = gaussian_bump(n, 1, sigma) + np.random.default_rng(seed_t).normal(0.0, 1e-3, size=shp)
    fill_periodic(lam, 1)
    fill_periodic(T0, 1)
    dt = cfl / float(lam[1:-1, 1:-1, 1:-1].max())
    return np.ascontiguousarray(lam), np.ascontiguousarray(T0), dt


def deep_inputs(n, seeds=(3, 4, 5, 6), frac=0.05):
    """a (SVol), b, c (XVol) full windows and the mask point list (interior-relative, x,y,z)."""
    n = (n, n, n) if np.isscalar(n) else tuple(n)
    shp = window_shape(n, 1)
    a = np.random.default_rng(seeds[0]).uniform(-1.0, 1.0, size=shp)
    b = np.random.default_rng(seeds[1]).uniform(-1.0, 1.0, size=shp)
    c = np.random.default_rng(seeds[2]).uniform(-1.0, 1.0, size=shp)
    pick = np.random.default_rng(seeds[3]).random(size=(n[2], n[1], n[0])) < frac
    zz, yy, xx = np.meshgrid(np.arange(n[2]), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    edge = (xx == 0) | (xx == n[0] - 1) | (yy == 0) | (yy == n[1] - 1) | (zz == 0) | (zz == n[2] - 1)
    sel = pick | edge
    pts = np.stack([xx[sel], yy[sel], zz[sel]], axis=1).astype(np.int32)
    return a, b, c, np.ascontiguousarray(pts)


def mask_bits_from_points(pts, n, g=1):
    """Bit-packed 32-bit mask words over the ghosted window (bit = flat % 32, x fastest)."""
    n = (n, n, n) if np.isscalar(n) else tuple(n)
    gx, gy, gz = n[0] + 2 * g, n[1] + 2 * g, n[2] + 2 * g
    total = gx * gy * gz
    words = np.zeros((total + 31) // 32, dtype=np.uint32)
    flat = (pts[:, 0] + g) + gx * ((pts[:, 1] + g) + gy * (pts[:, 2] + g))
    np.bitwise_or.at(words, flat // 32, (np.uint32(1) << (flat % 32).astype(np.uint32)))
    return words


def patch_shapes(count=512, seed=7, lo=16, hi=96):
    return np.random.default_rng(seed).integers(lo, hi + 1, size=(count, 3)).astype(np.int32)


def patch_inputs(shapes, seed=7, cfl=0.15):
    """Per patch: (lambda scalar, T0 window (sigma = min edge/6), dt = cfl/lambda)."""
    rng = np.random.default_rng(seed + 1000)
    out = []
    for s in shapes:
        lam = float(rng.uniform(0.5, 1.5))
        n = (int(s[0]), int(s[1]), int(s[2]))
        T0 = gaussian_bump(n, 1, sigma=min(n) / 6.0) + rng.normal(0.0, 1e-3, size=window_shape(n, 1))
        fill_periodic(T0, 1)
        out.append((lam, np.ascontiguousarray(T0), cfl / lam))
    return out


def adjoint_inputs(n, seed=8, cfl=0.15):
    lam, T0, dt = heat_inputs(n, cfl=cfl)
    nn = (n, n, n) if np.isscalar(n) else tuple(n)
    x = np.arange(-1, nn[0] + 1) + 0.5
    pert = 1.0 + 0.1 * np.sin(2.0 * np.pi * x / nn[0] + np.random.default_rng(seed).uniform(0, 2 * np.pi))
    lam_t = lam * pert[None, None, :]
    fill_periodic(lam_t, 1)
    return lam, T0, dt, np.ascontiguousarray(lam_t)


def transport_inputs(n, seed=10, modes=4, nu=0.05):
    """phi0, u (XVol), v (YVol), w (ZVol), lambda; windows with 2 ghosts, periodic.

    The face velocities are the discrete curl of a vector potential A sampled on cell edges,
    so Grad_{X->S}(u) + Grad_{Y->S}(v) + Grad_{Z->S}(w) vanishes up to rounding.
    """
    g = 2
    shp = window_shape(n, g)
    rng = np.random.default_rng(seed)
    zz, yy, xx = np.meshgrid(*(np.arange(-g, n + g, dtype=np.float64),) * 3, indexing="ij")
    A = [np.zeros(shp) for _ in range(3)]
    for _ in range(modes):
        k = rng.integers(1, 4, size=3) * rng.choice([-1, 1], size=3)
        amp = rng.normal(size=3)
        ph = rng.uniform(0, 2 * np.pi)
        arg = 2 * np.pi * (k[0] * xx + k[1] * yy + k[2] * zz) / n + ph
        for d in range(3):
            A[d] += amp[d] * np.sin(arg)
    Ax, Ay, Az = A

    def dfwd(f, axis):  # forward difference f[i+1]-f[i] along numpy axis
        return np.roll(f, -1, axis=axis) - f

    # u on x-faces: dAz/dy - dAy/dz ; v: dAx/dz - dAz/dx ; w: dAy/dx - dAx/dy
    u = dfwd(Az, 1) - dfwd(Ay, 0)
    v = dfwd(Ax, 0) - dfwd(Az, 2)
    w = dfwd(Ay, 2) - dfwd(Ax, 1)
    umax = max(np.abs(u).max(), np.abs(v).max(), np.abs(w).max())
    u, v, w = (q / umax for q in (u, v, w))
    for q in (u, v, w):
        fill_periodic(q, g)
    lam = rng.uniform(0.5, 1.5, size=shp)
    fill_periodic(lam, g)
    phi = gaussian_bump(n, g, sigma=n / 8.0)
    fill_periodic(phi, g)
    dt = 0.4  # CFL 0.4 with |u| <= 1 and unit spacing
    return (np.ascontiguousarray(phi), np.ascontiguousarray(u), np.ascontiguousarray(v),
            np.ascontiguousarray(w), np.ascontiguousarray(lam), dt, nu)


def transport_inputs_device(n, seed=10, modes=4, nu=0.05, device="cuda"):
    """transport_inputs built with torch on the GPU (same construction; for the full-size runs,
    where numpy on the host would take minutes).  Returns torch float64 tensors."""
    import torch

    g = 2
    rng = np.random.default_rng(seed)
    ax = torch.arange(-g, n + g, dtype=torch.float64, device=device)
    zz, yy, xx = torch.meshgrid(ax, ax, ax, indexing="ij")
    A = [torch.zeros_like(xx) for _ in range(3)]
    for _ in range(modes):
        k = rng.integers(1, 4, size=3) * rng.choice([-1, 1], size=3)
        amp = rng.normal(size=3)
        ph = rng.uniform(0, 2 * np.pi)
        arg = (2 * np.pi / n) * (float(k[0]) * xx + float(k[1]) * yy + float(k[2]) * zz) + ph
        s = torch.sin(arg)
        for d in range(3):
            A[d] += float(amp[d]) * s
        del arg, s
    Ax, Ay, Az = A

    def dfwd(f, axis):
        return torch.roll(f, -1, dims=axis) - f

    u = dfwd(Az, 1) - dfwd(Ay, 0)
    v = dfwd(Ax, 0) - dfwd(Az, 2)
    w = dfwd(Ay, 2) - dfwd(Ax, 1)
    del A, Ax, Ay, Az
    umax = max(float(u.abs().max()), float(v.abs().max()), float(w.abs().max()))
    u, v, w = u / umax, v / umax, w / umax
    lam = torch.from_numpy(rng.uniform(0.5, 1.5, size=(n + 2 * g,) * 3)).to(device)
    r2 = ((xx + 0.5 - n / 2.0) ** 2 + (yy + 0.5 - n / 2.0) ** 2 + (zz + 0.5 - n / 2.0) ** 2)
    phi = torch.exp(-r2 / (2.0 * (n / 8.0) ** 2))
    return phi.contiguous(), u.contiguous(), v.contiguous(), w.contiguous(), lam.contiguous(), 0.4, nu


# ----------------------------------------------------------------------------- particles
def particle_window(n, g, field="svol", bcx=False):
    """Allocation (= window, ghosts included) of an SVol or XVol cell field with g ghost cells
    (plus the +x boundary cell of an XVol with a boundary there), and its ghost cells on the -
    faces after limit_by_extent (0 on an axis of extent 1).  Returns (glob xyz, ngm xyz)."""
    n = tuple(n)
    glob, ngm = [], []
    for a in range(3):
        if n[a] > 1:
            glob.append(n[a] + 2 * g + (1 if (a == 0 and bcx and field == "xvol") else 0))
            ngm.append(g)
        else:
            glob.append(1)
            ngm.append(0)
    return tuple(glob), tuple(ngm)


def particle_inputs(n, g, nparticles, axes=7, spacing=(1.0, 1.0, 1.0), low=(0.5, 0.5, 0.5),
                    size_range=(0.3, 2.5), seed=11, spill=False, field="svol", bcx=False):
    """Seeded inputs of one particle <-> cell case.

    Cell values ~ U(-1, 1) over the whole allocation; particle values ~ U(0.5, 2); particle
    edges ~ U(size_range) x the smallest spacing of the axes in use.  Along each axis in use the
    centres are uniform such that every box lies inside the window, or (spill=True) such that a
    box may stick out of either end by up to 0.9 of a cell (the reference's own behaviour is
    defined there).  Axes not in use get coordinates 0.  `spacing` / `low` are the operator's
    state after its constructor (spacing > 0)."""
    rng = np.random.default_rng(seed)
    glob, ngm = particle_window(n, g, field, bcx)
    cell = rng.uniform(-1.0, 1.0, size=(glob[2], glob[1], glob[0]))
    on = [(axes >> a) & 1 for a in range(3)]
    dmin = min(spacing[a] for a in range(3) if on[a]) if any(on) else 1.0
    size = rng.uniform(size_range[0], size_range[1], nparticles) * dmin
    pos = []
    for a in range(3):
        if not on[a]:
            pos.append(np.zeros(nparticles))
            continue
        d = spacing[a]
        face = low[a] - d * ngm[a] - d / 2
        span = glob[a] * d
        r = size / 2
        u = rng.uniform(0.0, 1.0, nparticles)
        if spill:
            lo_c, hi_c = face - 0.9 * d + r, face + span + 0.9 * d - r
        else:
            lo_c, hi_c = face + r, face + span - r
        pos.append(lo_c + u * np.maximum(hi_c - lo_c, 0.0))
    pval = rng.uniform(0.5, 2.0, nparticles)
    return dict(glob=np.array(glob), ngm=np.array(ngm), cell=cell, px=pos[0], py=pos[1], pz=pos[2],
                psize=size, pval=pval, axes=axes, spacing=np.array(spacing, dtype=float),
                low=np.array(low, dtype=float))
