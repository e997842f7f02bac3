"""The integer-pipe FP64 exp and sin (nebo_fastmath_eval, the functions of the deep chain)
against CUDA's own (torch's) exp and sin, in ulps."""
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
