"""Device hmath == host hmath, bit for bit (the property the bitwise model
parity rests on), over random and edge-case inputs."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

_dp = C.POINTER(C.c_double)


def _eval(lib, op, where, x, y=None):
    x = np.ascontiguousarray(x, np.float64)
    y = None if y is None else np.ascontiguousarray(y, np.float64)
    out = np.empty_like(x)
    rc = lib.mhm_hmath_eval(op, where, len(x), x.ctypes.data_as(_dp),
                            None if y is None else y.ctypes.data_as(_dp), out.ctypes.data_as(_dp))
    assert rc == 0
    return out


def _inputs(n=1 << 20, seed=0):
    rng = np.random.default_rng(seed)
    x = np.exp(rng.uniform(-700, 700, n))
    x[:64] = [0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 5e-324, 2.2250738585072014e-308,
              0.5, 2.0, 0.7070, 1.4142, 1 - 2**-53, 1 + 2**-52, 1e-300, 1e300, 1.7976931348623157e308] + \
        list(rng.uniform(0.99, 1.01, 46))
    e = rng.uniform(-750, 712, n)
    e[:16] = [0.0, -0.0, 1.0, -1.0, np.inf, -np.inf, np.nan, 708.0, -708.0, 709.78, -745.13, -746.0, 710.0,
              1e-300, -1e-300, 2**-30]
    y = rng.uniform(0.0, 3.0, n)
    return x, e, y


def test_device_equals_host(lib):
    x, e, y = _inputs()
    xp = np.where(np.isfinite(x), np.abs(x), 1.0) % 1000.0
    b = np.random.default_rng(9).integers(0, 2**64, len(x), dtype=np.uint64).view(np.float64)
    for op, arg, yy in ((0, x, None), (1, e, None), (2, xp, y), (3, x, b)):
        d = _eval(lib, op, 1, arg, yy)
        h = _eval(lib, op, 0, arg, yy)
        same = (d.view(np.uint64) == h.view(np.uint64)) | (np.isnan(d) & np.isnan(h))
        assert same.all(), (op, np.flatnonzero(~same)[:5])
