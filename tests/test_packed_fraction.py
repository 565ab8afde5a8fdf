"""The two facts behind the cell chain's packed runoff fractions, checked on
the host with the library's own log / exp / division (hmath.h and fp64i.h
through mhm_hmath_eval, host side) and IEEE double arithmetic.

The soil-moisture update of one horizon (src/mHM/mo_soil_moisture.f90:230-245)
is, for SM <= SMs,

    frac   = exp(beta * log(SM / SMs))       (0 when SM <= eps)
    tmp    = pin * (1 - frac)
    filled = SM + tmp
    infil  = pin + (SM - SMs)  if filled > SMs  else  pin + (-tmp)
    SM     = SMs               if filled > SMs  else  filled

(1) With SMs finite and beta finite and > 0, frac lies in [0, 1] for every
eps < SM <= SMs.  (2) With pin = +0 and frac in [0, 1] the update gives
infil = +0 and leaves SM unchanged whatever frac is, so a cell whose
effective precipitation is +0 needs none of its fractions.  Parameters outside
(1) can make frac NaN or > 1, which is why the kernel evaluates them as
always.
"""
import ctypes as C

import numpy as np

EPS = np.finfo(np.float64).eps
_dp = C.POINTER(C.c_double)


def _hm(lib, op, x, y=None):
    x = np.ascontiguousarray(x, np.float64)
    y = None if y is None else np.ascontiguousarray(y, np.float64)
    out = np.empty_like(x)
    rc = lib.mhm_hmath_eval(op, 0, len(x), x.ctypes.data_as(_dp),
                            None if y is None else y.ctypes.data_as(_dp), out.ctypes.data_as(_dp))
    assert rc == 0
    return out


def _frac(lib, sm, sms, beta):
    """exp(beta * log(SM / SMs)) as the kernel and the oracle evaluate it
    (a huge beta takes the product to -inf, and the fraction to 0)."""
    with np.errstate(over="ignore"):
        x = beta * _hm(lib, 0, _hm(lib, 3, sm, sms))
    return _hm(lib, 1, x)


def _horizon(pin, sm, sms, frac):
    tmp = pin * (1.0 - frac)
    filled = sm + tmp
    over = filled > sms
    infil = pin + np.where(over, sm - sms, -tmp)
    return infil, np.where(over, sms, filled)


def _samples(rng, n):
    sms = 10.0 ** rng.uniform(-300, 300, n)
    sms[: n // 10] = np.finfo(np.float64).max
    sm = np.minimum(sms, np.maximum(EPS * (1 + rng.random(n)), sms * rng.random(n)))
    sm[n // 10: n // 5] = sms[n // 10: n // 5]                 # SM == SMs: log 1 = 0
    sm[n // 5: n // 4] = EPS * 1.5                             # SM just above eps
    beta = 10.0 ** rng.uniform(-320, 300, n)
    beta[: n // 20] = 5e-324
    beta[n // 20: n // 10] = np.finfo(np.float64).max
    keep = (sm > EPS) & (sm <= sms)                            # the branch the fraction is taken in
    return sm[keep], sms[keep], beta[keep]


def test_fraction_bounded_for_finite_positive_parameters(lib):
    rng = np.random.default_rng(71)
    sm, sms, beta = _samples(rng, 400_000)
    fr = _frac(lib, sm, sms, beta)
    assert not np.isnan(fr).any()
    assert (fr >= 0.0).all() and (fr <= 1.0).all()


def test_zero_input_ignores_the_fraction():
    rng = np.random.default_rng(72)
    n = 200_000
    sms = 10.0 ** rng.uniform(-300, 300, n)
    sm = np.minimum(sms, np.maximum(EPS * (1 + rng.random(n)), sms * rng.random(n)))
    pin = np.zeros(n)                                   # +0
    ref_infil, ref_sm = _horizon(pin, sm, sms, np.zeros(n))
    assert (ref_infil.view(np.uint64) == 0).all()       # +0, not -0
    assert np.array_equal(ref_sm.view(np.uint64), sm.view(np.uint64))
    for fr in (np.ones(n), rng.random(n), np.full(n, 0.5), np.nextafter(np.ones(n), 0.0)):
        infil, smn = _horizon(pin, sm, sms, fr)
        assert np.array_equal(infil.view(np.uint64), ref_infil.view(np.uint64))
        assert np.array_equal(smn.view(np.uint64), ref_sm.view(np.uint64))


def test_parameters_outside_the_bound_change_the_update(lib):
    """Why those cells are evaluated as always: beta = 0 with SMs = inf gives
    0 * log(0) = NaN, and a negative beta a fraction above 1."""
    with np.errstate(invalid="ignore"):
        fr = _frac(lib, np.array([1.0]), np.array([np.inf]), np.array([0.0]))
        assert np.isnan(fr).all()
        infil, _ = _horizon(np.zeros(1), np.array([1.0]), np.array([np.inf]), fr)
    assert np.isnan(infil).all()
    fr = _frac(lib, np.array([0.5]), np.array([1.0]), np.array([-0.4]))
    assert (fr > 1.0).all()
