"""The integer-pipe FP64 exp and sin (nebo_fastmath_eval, the functions of the deep chain)
against CUDA's own (torch's) exp and sin, in ulps."""
import ctypes
import zlib

import numpy as np
import pytest

import spatialops_gb300 as N

pytestmark = pytest.mark.gpu


def _ulps(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    ia = a.view(np.int64)
    ib = b.view(np.int64)
    ia = np.where(ia < 0, np.int64(-0x8000000000000000) - ia, ia)
    ib = np.where(ib < 0, np.int64(-0x8000000000000000) - ib, ib)
    return np.abs(ia - ib)


def _inputs(rng, lo, hi, n=1 << 20):
    return rng.uniform(lo, hi, size=n)


@pytest.mark.parametrize("fn,lo,hi", [("exp", -1, 1), ("exp", -707.9, 707.9), ("exp", -1e-6, 1e-6),
                                      ("exp", -40, 40), ("sin", -1, 1), ("sin", -100, 100), ("sin", -1e5, 1e5),
                                      ("sin", -1e-8, 1e-8), ("sin", -1048575, 1048575), ("sin", -0.05, 0.05)])
def test_within_two_ulp_of_cuda(fn, lo, hi):
    import torch

    rng = np.random.default_rng(zlib.crc32(repr((fn, lo, hi)).encode()))
    x = torch.from_numpy(_inputs(rng, lo, hi)).cuda()
    got = N.fastmath_eval(fn, x).cpu().numpy()
    ref = (torch.exp(x) if fn == "exp" else torch.sin(x)).cpu().numpy()
    u = _ulps(got, ref)
    assert u.max() <= 2, (fn, lo, hi, int(u.max()))
    assert u.mean() < 0.5


def test_special_values():
    import torch

    x = torch.tensor([0.0, -0.0, 1.0, -1.0, 709.0, -745.0, 800.0, float("inf"), -float("inf"), float("nan"),
                      np.pi, -np.pi, np.pi / 2, 3 * np.pi / 2, 2.0 ** 21, 1e300], dtype=torch.float64).cuda()
    for fn, ref in (("exp", torch.exp), ("sin", torch.sin)):
        got = N.fastmath_eval(fn, x).cpu().numpy()
        r = ref(x).cpu().numpy()
        same = (got == r) | (np.isnan(got) & np.isnan(r)) | (_ulps(got, r) <= 2)
        assert same.all(), (fn, got, r)


def test_sin_near_multiples_of_pi():
    """k a multiple of 64: the result is +-sin r with r possibly tiny (the four-part pi/64 branch)."""
    import torch

    j = np.arange(1, 333000, 7, dtype=np.float64)
    base = j * np.pi
    x = np.concatenate([base, np.nextafter(base, np.inf), np.nextafter(base, -np.inf), -base,
                        base * 0.5 + 1e-3, np.array([0.0, -0.0, 1e-300, -1e-300, 5e-324])])
    xt = torch.from_numpy(x).cuda()
    got = N.fastmath_eval("sin", xt).cpu().numpy()
    ref = torch.sin(xt).cpu().numpy()
    u = _ulps(got, ref)
    assert u.max() <= 2, (int(u.max()), x[int(np.argmax(u))])
    assert (np.signbit(got[-4:]) == np.signbit(x[-4:])).all()


def _quotients(fn, a, b):
    import torch

    import spatialops_gb300 as S

    x = torch.from_numpy(np.stack([a, b], axis=1).ravel().copy()).cuda()
    y = torch.empty(len(a), dtype=torch.float64, device="cuda")
    S._check(S.lib().nebo_fastmath_eval(fn, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()),
                                        len(a), S._stream()))
    torch.cuda.synchronize()
    return y.cpu().numpy()


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_reciprocal_quotient_is_correctly_rounded(seed):
    # the particle operators' a / b from RN(1/b) and two FMA corrections against the division,
    # bit for bit: random mantissas over wide exponent ranges, the operators' own value ranges
    # (products of overlaps over particle volumes), exact quotients, signed zeros, and operands
    # outside the corrected path's range (division fallback)
    rng = np.random.default_rng(seed)
    n = 4_000_000
    a = rng.uniform(1, 2, n) * np.exp2(rng.integers(-60, 60, n))
    b = rng.uniform(1, 2, n) * np.exp2(rng.integers(-60, 60, n))
    a[: n // 8] = rng.uniform(0, 1, n // 8) ** 3                   # overlap products in [0, 1]
    b[: n // 8] = rng.uniform(0.1, 3.0, n // 8) ** 3               # particle volumes
    k = rng.integers(1, 1 << 20, n // 8).astype(np.float64)
    a[n // 8: n // 4] = k * b[n // 8: n // 4]                      # exact integer quotients (where exact)
    a[n // 4: n // 4 + 1000] = 0.0
    a[n // 4 + 1000: n // 4 + 2000] = -0.0
    a[n // 4 + 2000: n // 4 + 3000] = np.exp2(-900.0) * rng.uniform(1, 2, 1000)  # fallback ranges
    b[n // 4 + 3000: n // 4 + 4000] = np.exp2(600.0)
    neg = rng.random(n) < 0.3
    a[neg] = -a[neg]
    fast = _quotients(2, a, b)
    div = _quotients(3, a, b)
    assert np.array_equal(fast.view(np.uint64), div.view(np.uint64))
    assert np.array_equal(div, a / b)  # and the host's correctly rounded division
