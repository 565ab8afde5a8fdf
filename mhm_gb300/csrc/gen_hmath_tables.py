#!/usr/bin/env python3
"""Generate ``hmath_tables.h``: the lookup tables of the table-driven FP64
``log`` and ``exp`` in ``hmath.h``.

Method (named, published): P. T. P. Tang, "Table-driven implementation of the
exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989,
and "Table-driven implementation of the logarithm function in IEEE
floating-point arithmetic", ACM TOMS 16(4), 1990.  The reduction points and the
polynomial (plain Taylor coefficients of log1p / expm1) are this project's own
choices; every constant below is computed here with mpmath at 200 bits and
rounded to the nearest double.

log:  x = 2^k * z, z in [OFF, 2*OFF) with OFF = 0x3FE6A00000000000 (~0.7070);
      256 sub-intervals indexed by the top 8 bits of (bits(x) - OFF) below the
      exponent.  Each sub-interval has a 9-significant-bit reciprocal ``invc``
      so that r = z*invc - 1 is EXACT in one fma (|r| < 2^-8 and z*invc has at
      most 62 significant bits), and logc = -log(invc) stored as a
      double-double whose high part lies on the 2^-42 grid, so that
      k*LN2_HI + logc_hi is exact as well.
exp:  x = (k/128)*ln2 + r, |r| <= ln2/256; table of 2^(j/128), j=0..127, as a
      double-double.

Run:  python gen_hmath_tables.py > hmath_tables.h
"""
import struct

import mpmath as mp

mp.mp.prec = 200


def d2b(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def b2d(b: int) -> float:
    return struct.unpack("<d", struct.pack("<Q", b & 0xFFFFFFFFFFFFFFFF))[0]


def to_double(v) -> float:
    """Round an mpmath number to the nearest double (round-half-even)."""
    return float(mp.mpf(v))


def round_to_grid(v, quantum):
    return mp.nint(v / quantum) * quantum


def round_sig_bits(v, bits):
    """Round positive v to `bits` significant bits."""
    e = mp.floor(mp.log(v, 2))
    q = mp.mpf(2) ** (e - bits + 1)
    return mp.nint(v / q) * q


def hexd(x: float) -> str:
    return "0x%016xULL" % d2b(x)


OFF = 0x3FE6A00000000000
LOG_NBITS = 8
LOG_N = 1 << LOG_NBITS
LOG_SHIFT = 52 - LOG_NBITS
GRID = mp.mpf(2) ** -42


def log_table():
    rows = []
    one_bits = d2b(1.0)
    for j in range(LOG_N):
        lo_b = OFF + (j << LOG_SHIFT)
        hi_b = OFF + ((j + 1) << LOG_SHIFT) - 1
        zlo, zhi = mp.mpf(b2d(lo_b)), mp.mpf(b2d(hi_b))
        c = (zlo + zhi) / 2
        if lo_b <= one_bits <= hi_b + 1:
            # the two sub-intervals that touch 1.0 use invc = 1 exactly, so
            # r = z - 1 and log is accurate near 1
            invc = mp.mpf(1)
        else:
            invc = round_sig_bits(1 / c, 9)
        r_lo = zlo * invc - 1
        r_hi = zhi * invc - 1
        rmax = max(abs(r_lo), abs(r_hi))
        assert rmax < mp.mpf(2) ** -8, (j, rmax)
        logc = -mp.log(invc)
        lhi = round_to_grid(logc, GRID)
        llo = logc - lhi
        lhi_d = to_double(lhi)
        assert mp.mpf(lhi_d) == lhi
        llo_d = to_double(llo)
        # Fast2Sum(w, r) in hmath.h needs |logc_hi| >= |r| whenever logc_hi != 0
        if lhi != 0:
            assert abs(lhi) >= rmax, (j, lhi, rmax)
        rows.append((to_double(invc), lhi_d, llo_d))
    return rows


def exp_table():
    rows = []
    for j in range(128):
        t = mp.mpf(2) ** (mp.mpf(j) / 128)
        thi = to_double(t)
        tlo = to_double(t - mp.mpf(thi))
        rows.append((thi, tlo))
    return rows


def main():
    ln2 = mp.log(2)
    ln2_hi = round_to_grid(ln2, GRID)  # 42-bit: k*LN2_HI exact for |k| < 2^11
    ln2_lo = to_double(ln2 - ln2_hi)
    ln2n = ln2 / 128
    ln2n_hi = round_to_grid(ln2n, mp.mpf(2) ** -(7 + 35))  # kd*LN2N_HI exact for |kd| < 2^18
    ln2n_lo = to_double(ln2n - ln2n_hi)
    inv_ln2n = to_double(128 / ln2)
    print("/* Generated by gen_hmath_tables.py -- do not edit by hand. */")
    print("/* Tables for the table-driven FP64 log/exp of hmath.h (Tang 1989/1990 method). */")
    print("#pragma once")
    print("#define HM_LOG_OFF 0x%016xULL" % OFF)
    print("#define HM_LOG_NBITS %d" % LOG_NBITS)
    print("#define HM_LN2_HI %s /* %r */" % (hexd(to_double(ln2_hi)), to_double(ln2_hi)))
    print("#define HM_LN2_LO %s /* %r */" % (hexd(ln2_lo), ln2_lo))
    print("#define HM_EXP_INVLN2N %s /* 128/ln2 = %r */" % (hexd(inv_ln2n), inv_ln2n))
    print("#define HM_EXP_LN2N_HI %s /* %r */" % (hexd(to_double(ln2n_hi)), to_double(ln2n_hi)))
    print("#define HM_EXP_LN2N_LO %s /* %r */" % (hexd(ln2n_lo), ln2n_lo))
    # Taylor coefficients of log1p(r) = r + r^2*(c2 + r*(c3 + ... + r*c7))
    for n in range(2, 8):
        v = to_double(mp.mpf((-1) ** (n + 1)) / n)
        print("#define HM_LOG_C%d %s /* %r */" % (n, hexd(v), v))
    # Taylor coefficients of expm1(r) = r + r^2*(e2 + r*(e3 + r*(e4 + r*e5)))
    for n in range(2, 6):
        v = to_double(1 / mp.factorial(n))
        print("#define HM_EXP_C%d %s /* %r */" % (n, hexd(v), v))
    lt = log_table()
    print("/* log table: {invc, logc_hi, logc_lo} x %d, as IEEE-754 bit patterns */" % LOG_N)
    print("#define HM_LOG_TABLE_INIT { \\")
    for invc, lhi, llo in lt:
        print("  %s, %s, %s, \\" % (hexd(invc), hexd(lhi), hexd(llo)))
    print("}")
    et = exp_table()
    print("/* exp table: {2^(j/128) hi, lo} x 128, as IEEE-754 bit patterns */")
    print("#define HM_EXP_TABLE_INIT { \\")
    for thi, tlo in et:
        print("  %s, %s, \\" % (hexd(thi), hexd(tlo)))
    print("}")
    fixed_point_tables(lt)


def q(v, frac_bits):
    """Round v * 2^frac_bits to the nearest integer (mpmath)."""
    return int(mp.nint(mp.mpf(v) * mp.mpf(2) ** frac_bits))


def limbs128(n):
    """Signed 128-bit integer -> (hi as int64 two's complement, lo as uint64)."""
    n &= (1 << 128) - 1
    return (n >> 64), n & ((1 << 64) - 1)


def fixed_point_tables(lt):
    """Integer-pipe variants: every quantity as a fixed-point integer.
    Q116 = signed 128-bit integer scaled by 2^-116, Q64/Q63 = 64-bit."""
    print("/* ---- fixed-point (integer pipe) log/exp ---- */")
    ln2 = mp.log(2)
    hi, lo = limbs128(q(ln2, 116))
    print("#define HM_FX_LN2_Q116_HI 0x%016xULL" % hi)
    print("#define HM_FX_LN2_Q116_LO 0x%016xULL" % lo)
    hi, lo = limbs128(q(ln2 / 128, 116))
    print("#define HM_FX_LN2N_Q116_HI 0x%016xULL" % hi)
    print("#define HM_FX_LN2N_Q116_LO 0x%016xULL" % lo)
    print("#define HM_FX_INVLN2N_Q54 0x%016xULL /* round(128/ln2 * 2^54) */" % q(128 / ln2, 54))
    print("#define HM_FX_INVLN10_Q64 0x%016xULL /* round(2^64 / ln10) */" % q(1 / mp.log(10), 64))
    # log1p(r) = r * (1 + r * q(r)), q = -1/2 + r/3 - r^2/4 + r^3/5 - r^4/6 + r^5/7 (Q63)
    for n in range(2, 8):
        v = q(mp.mpf((-1) ** (n + 1)) / n, 63)
        print("#define HM_FX_LOG_C%d ((int64_t)0x%016xULL)" % (n, v & ((1 << 64) - 1)))
    # expm1(r) = r + r^2 * (1/2 + r/6 + r^2/24 + r^3/120 + r^4/720) (Q63)
    for n in range(2, 7):
        v = q(1 / mp.factorial(n), 63)
        print("#define HM_FX_EXP_C%d ((int64_t)0x%016xULL)" % (n, v))
    # log table: A (invc * 2^9 for z >= 1, invc * 2^8 for z < 1) and -log(invc) in Q116
    one_idx = None
    print("/* log: {A, logc Q116 hi, logc Q116 lo} x 256 */")
    print("#define HM_FX_LOG_TABLE_INIT { \\")
    for j, (invc, _, _) in enumerate(lt):
        zlo_bits = OFF + (j << LOG_SHIFT)
        scale = 9 if (zlo_bits >> 52) >= 0x3FF else 8
        A = mp.mpf(invc) * mp.mpf(2) ** scale
        assert A == mp.nint(A), (j, invc)
        logc = -mp.log(mp.mpf(invc))
        hi, lo = limbs128(q(logc, 116))
        print("  0x%016xULL, 0x%016xULL, 0x%016xULL, \\" % (int(A), hi, lo))
    print("}")
    print("/* exp: 2^(j/128) in Q63, x 128 */")
    print("#define HM_FX_EXP_TABLE_INIT { \\")
    for j in range(128):
        v = q(mp.mpf(2) ** (mp.mpf(j) / 128), 63)
        assert v < (1 << 64)
        print("  0x%016xULL, \\" % v)
    print("}")


if __name__ == "__main__":
    main()
