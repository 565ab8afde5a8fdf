"""Accuracy of the shared elementary functions (hmath.h) and exactness of the
integer-pipe division (fp64i.h), evaluated on the host through the C ABI.
log/exp/pow: within 1 ulp of the C library and below 0.6 ulp of the exact
value (mpmath, 100 digits); division: identical to IEEE division."""
import ctypes as C

import numpy as np
import pytest

_dp = C.POINTER(C.c_double)


def _eval(lib, op, x, y=None, where=0):
    x = np.ascontiguousarray(x, np.float64)
    y = None if y is None else np.ascontiguousarray(y, np.float64)
    out = np.empty_like(x)
    rc = lib.mhm_hmath_eval(op, where, len(x), x.ctypes.data_as(_dp),
                            None if y is None else y.ctypes.data_as(_dp), out.ctypes.data_as(_dp))
    assert rc == 0
    return out


def _ulp_diff(a, b):
    a = a.view(np.int64)
    b = b.view(np.int64)
    return np.abs(a - b)


def test_log_exp_pow_vs_libm(lib):
    rng = np.random.default_rng(1)
    x = np.exp(rng.uniform(-740, 709, 1_000_000))
    x[:200_000] = 1.0 + rng.uniform(-1e-3, 1e-3, 200_000)
    assert _ulp_diff(_eval(lib, 0, x), np.log(x)).max() <= 1
    e = rng.uniform(-745, 709, 1_000_000)
    e[:200_000] = rng.uniform(-1e-3, 1e-3, 200_000)
    assert _ulp_diff(_eval(lib, 1, e), np.exp(e)).max() <= 1
    b = rng.uniform(0, 500, 500_000)
    p = rng.uniform(0, 3, 500_000)
    assert _ulp_diff(_eval(lib, 2, b, p), np.power(b, p)).max() <= 1


def test_vs_mpmath(lib):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 100
    rng = np.random.default_rng(2)
    xs = np.concatenate([np.exp(rng.uniform(-700, 700, 3000)), 1 + rng.uniform(-1e-6, 1e-6, 500)])
    worst = 0.0
    for op, arg, f in ((0, xs, mp.log), (1, rng.uniform(-700, 700, 3000), mp.exp)):
        got = _eval(lib, op, arg)
        for g, v in zip(got, arg):
            ex = f(mp.mpf(float(v)))
            ulp = np.spacing(abs(float(ex)))
            worst = max(worst, abs(float((mp.mpf(float(g)) - ex) / ulp)))
    assert worst < 0.6, worst


def test_special_values(lib):
    x = np.array([0.0, -0.0, -1.0, np.inf, np.nan, 1.0, 5e-324])
    lg = _eval(lib, 0, x)
    assert lg[0] == -np.inf and lg[1] == -np.inf and np.isnan(lg[2]) and lg[3] == np.inf
    assert np.isnan(lg[4]) and lg[5] == 0.0 and lg[6] == np.log(5e-324)
    ex = _eval(lib, 1, np.array([0.0, np.inf, -np.inf, np.nan, 710.0, -746.0, -745.0, 709.78]))
    assert ex[0] == 1.0 and ex[1] == np.inf and ex[2] == 0.0 and np.isnan(ex[3])
    assert ex[4] == np.inf and ex[5] == 0.0 and ex[6] == np.exp(-745.0) and ex[7] == np.exp(709.78)
    pw = _eval(lib, 2, np.array([0.0, 1.0, -1.0, 0.25, 2.0]), np.array([2 / 3, 3.3, 0.5, 0.0, 1.5]))
    assert pw[0] == 0.0 and pw[1] == 1.0 and np.isnan(pw[2]) and pw[3] == 1.0 and pw[4] == 2.0 ** 1.5


def test_division_exact(lib):
    rng = np.random.default_rng(3)
    n = 2_000_000
    a = rng.integers(0, 2**64, n, dtype=np.uint64).view(np.float64)
    b = rng.integers(0, 2**64, n, dtype=np.uint64).view(np.float64)
    b[: n // 4] = rng.uniform(0.5, 2.0, n // 4)  # near-1 divisors
    b[n // 4: n // 2] = np.ldexp(1.0, rng.integers(-60, 60, n // 4))  # powers of two
    a[:1000] = 0.0
    spec = np.array([0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 5e-324, 1e-310, 1.7976931348623157e308])
    a = np.concatenate([a, np.repeat(spec, len(spec))])
    b = np.concatenate([b, np.tile(spec, len(spec))])
    with np.errstate(all="ignore"):
        ref = a / b
    got = _eval(lib, 3, a, b)
    same = (got.view(np.uint64) == ref.view(np.uint64)) | (np.isnan(got) & np.isnan(ref))
    assert same.all(), np.flatnonzero(~same)[:5]
