/*
 * hmath.h -- FP64 log / exp / pow shared bit-for-bit by host and device code.
 *
 * The mHM water-balance chain evaluates, per cell and time step, the power
 * laws of src/mHM/mo_canopy_interc.f90:117 ((I/Imax)**(2/3)),
 * src/mHM/mo_runoff.f90:139 (u**(1+alpha)) and the exp(b*log(x)) of
 * src/mHM/mo_soil_moisture.f90:233.  Storage thresholds branch on the results
 * thousands of times per run, so the device kernels and the CPU oracle use the
 * SAME elementary functions: this header.  Every operation is an IEEE-754
 * double operation with round-to-nearest, fused multiply-adds are written out
 * as fma() (compile host code with -ffp-contract=off and device code with
 * --fmad=false), so a host build and a device build return identical bits.
 *
 * Method: table-driven reduction after P. T. P. Tang (ACM TOMS 1989, exp;
 * ACM TOMS 1990, log) with Taylor polynomials; constants and tables are
 * generated by gen_hmath_tables.py (mpmath, 200 bits).  Accuracy (checked in
 * tests/test_hmath.py against mpmath): log and exp below 0.52 ulp, pow (log
 * carried as a double-double) below 1 ulp on the tested domain.
 *
 * Special values follow C99 Annex F for the cases the model can produce:
 * log(+-0) = -inf, log(x<0) = NaN, log(+inf) = +inf, log(NaN) = NaN;
 * exp(+inf) = +inf, exp(-inf) = 0, exp(NaN) = NaN, gradual underflow;
 * pow(x, y) = exp(y*log(x)) for x >= 0 (pow(0, y>0) = 0, pow(1, y) = 1),
 * NaN for x < 0.
 *
 * This file is plain C99 and CUDA C++; it is included by the CUDA kernels and
 * by the C oracle (as a shared math library, not as model code).
 */
#ifndef MHM_HMATH_H
#define MHM_HMATH_H

#include <stdint.h>
#include "hmath_tables.h"

#if defined(__CUDACC__)
#define HM_FN static __host__ __device__ __forceinline__
/* the large functions (log, exp, pow, div) are compiled out of line: one
 * copy per kernel keeps the instruction footprint inside the SM's
 * instruction cache (measured faster than inlining; -DHM_INLINE inlines) */
#if defined(HM_INLINE)
#define HM_FN_BIG HM_FN
#else
#define HM_FN_BIG static __host__ __device__ __noinline__
#endif
#else
#include <math.h>
#include <string.h>
#define HM_FN static inline
#define HM_FN_BIG static inline
#endif

#define HM_LOG_N (1 << HM_LOG_NBITS)

HM_FN double hm_b2d(uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __longlong_as_double((long long)b);
#else
    double d;
    memcpy(&d, &b, sizeof d);
    return d;
#endif
}

HM_FN uint64_t hm_d2b(double d)
{
#if defined(__CUDA_ARCH__)
    return (uint64_t)__double_as_longlong(d);
#else
    uint64_t b;
    memcpy(&b, &d, sizeof b);
    return b;
#endif
}

/* The bits of |x| (sign bit cleared), as an integer.  On the device the mask
 * is inline PTX: written in C, the compiler recognises "bits of a double AND
 * 0x7fff..." as an FP64 absolute value and issues it on the FP64 pipe, which
 * on this GPU is the scarce one (measured: one extra FP64 instruction per
 * masked operand). */
HM_FN uint64_t hm_abs_bits(uint64_t u)
{
#if defined(__CUDA_ARCH__)
    uint64_t r;
    asm("and.b64 %0, %1, 0x7fffffffffffffff;" : "=l"(r) : "l"(u));
    return r;
#else
    return u & 0x7fffffffffffffffULL;
#endif
}

/* Default tables.  Host code reads static arrays; device code reads the
 * __device__ copies unless a kernel passes its own (e.g. shared-memory) copy. */
static const uint64_t hm_log_tab_h[3 * HM_LOG_N] = HM_LOG_TABLE_INIT;
static const uint64_t hm_exp_tab_h[2 * 128] = HM_EXP_TABLE_INIT;
#if defined(__CUDACC__)
static __device__ const uint64_t hm_log_tab_d[3 * HM_LOG_N] = HM_LOG_TABLE_INIT;
static __device__ const uint64_t hm_exp_tab_d[2 * 128] = HM_EXP_TABLE_INIT;
#endif
#if defined(__CUDA_ARCH__)
#define HM_LOG_TAB hm_log_tab_d
#define HM_EXP_TAB hm_exp_tab_d
#else
#define HM_LOG_TAB hm_log_tab_h
#define HM_EXP_TAB hm_exp_tab_h
#endif

#define HM_SHIFT 0x1.8p52 /* 1.5 * 2^52: round-to-integer shifter */

/* log(x) as an unevaluated sum hi + lo (|lo| <= ulp(hi)).  ltab: 3*256 words. */
HM_FN void hm_log_dd_t(double x, const uint64_t *ltab, double *hi_out, double *lo_out)
{
    uint64_t u = hm_d2b(x);
    uint32_t top = (uint32_t)(u >> 32);
    int64_t kadj = 0;
    if (top - 0x00100000u >= 0x7ff00000u - 0x00100000u) {
        /* zero, subnormal, negative, inf or NaN */
        if (hm_abs_bits(u) == 0) {               /* +-0 */
            *hi_out = -HUGE_VAL;
            *lo_out = 0.0;
            return;
        }
        if (u == 0x7ff0000000000000ULL) {  /* +inf */
            *hi_out = x;
            *lo_out = 0.0;
            return;
        }
        if ((top >> 31) || (top & 0x7ff00000u) == 0x7ff00000u) { /* x < 0 or NaN */
            *hi_out = hm_b2d(0x7ff8000000000000ULL);
            *lo_out = 0.0;
            return;
        }
        /* positive subnormal: scale into the normal range */
        u = hm_d2b(x * 0x1p52);
        kadj = -52;
    }
    uint64_t tmp = u - HM_LOG_OFF;
    int64_t k = ((int64_t)tmp >> 52) + kadj;
    uint32_t i = (uint32_t)(tmp >> (52 - HM_LOG_NBITS)) & (HM_LOG_N - 1);
    double z = hm_b2d(u - (tmp & 0xfff0000000000000ULL));
    double invc = hm_b2d(ltab[3 * i]);
    double lhi = hm_b2d(ltab[3 * i + 1]);
    double llo = hm_b2d(ltab[3 * i + 2]);
    double r = fma(z, invc, -1.0);                          /* exact */
    double kd = hm_b2d(0x4338000000000000ULL + (uint64_t)k) - HM_SHIFT; /* exact */
    double w = fma(kd, hm_b2d(HM_LN2_HI), lhi);             /* exact */
    double t = w + r;                                       /* Fast2Sum: |w| >= |r| or w == 0 */
    double e = (w - t) + r;
    double r2 = r * r;
    double q = fma(r, hm_b2d(HM_LOG_C7), hm_b2d(HM_LOG_C6));
    q = fma(r, q, hm_b2d(HM_LOG_C5));
    q = fma(r, q, hm_b2d(HM_LOG_C4));
    q = fma(r, q, hm_b2d(HM_LOG_C3));
    q = fma(r, q, hm_b2d(HM_LOG_C2));
    double lo = fma(kd, hm_b2d(HM_LN2_LO), llo) + e;
    lo = fma(r2, q, lo);
    double hi = t + lo;
    *hi_out = hi;
    *lo_out = (t - hi) + lo;
}

HM_FN double hm_log_t(double x, const uint64_t *ltab)
{
    uint64_t u = hm_d2b(x);
    uint32_t top = (uint32_t)(u >> 32);
    if (top - 0x00100000u >= 0x7ff00000u - 0x00100000u) {
        double h, l;
        hm_log_dd_t(x, ltab, &h, &l);
        return h + l;
    }
    uint64_t tmp = u - HM_LOG_OFF;
    int64_t k = (int64_t)tmp >> 52;
    uint32_t i = (uint32_t)(tmp >> (52 - HM_LOG_NBITS)) & (HM_LOG_N - 1);
    double z = hm_b2d(u - (tmp & 0xfff0000000000000ULL));
    double invc = hm_b2d(ltab[3 * i]);
    double lhi = hm_b2d(ltab[3 * i + 1]);
    double llo = hm_b2d(ltab[3 * i + 2]);
    double r = fma(z, invc, -1.0);
    double kd = hm_b2d(0x4338000000000000ULL + (uint64_t)k) - HM_SHIFT;
    double w = fma(kd, hm_b2d(HM_LN2_HI), lhi);
    double t = w + r;
    double e = (w - t) + r;
    double r2 = r * r;
    double q = fma(r, hm_b2d(HM_LOG_C7), hm_b2d(HM_LOG_C6));
    q = fma(r, q, hm_b2d(HM_LOG_C5));
    q = fma(r, q, hm_b2d(HM_LOG_C4));
    q = fma(r, q, hm_b2d(HM_LOG_C3));
    q = fma(r, q, hm_b2d(HM_LOG_C2));
    double lo = fma(kd, hm_b2d(HM_LN2_LO), llo) + e;
    lo = fma(r2, q, lo);
    return t + lo;
}

/* exp(x + xt) where xt is a small correction (|xt| <= 2^-40 |x| or so). */
HM_FN double hm_exp_dd_t(double x, double xt, const uint64_t *etab)
{
    uint64_t u = hm_d2b(x);
    uint32_t atop = (uint32_t)(u >> 32) & 0x7fffffffu;
    int special = atop >= 0x40862000u; /* |x| >= 708, inf or NaN */
    if (special) {
        if (x != x)
            return x;
        if (x > 710.0)
            return HUGE_VAL;
        if (x < -746.0)
            return 0.0;
        xt = 0.0;
    }
    double t = fma(x, hm_b2d(HM_EXP_INVLN2N), HM_SHIFT);
    int32_t k = (int32_t)(uint32_t)hm_d2b(t);
    double kd = t - HM_SHIFT;
    double r = fma(kd, -hm_b2d(HM_EXP_LN2N_HI), x);
    r = fma(kd, -hm_b2d(HM_EXP_LN2N_LO), r);
    r = r + xt;
    uint32_t j = (uint32_t)k & 127u;
    int32_t m = k >> 7; /* floor(k / 128) */
    double thi = hm_b2d(etab[2 * j]);
    double tlo = hm_b2d(etab[2 * j + 1]);
    double r2 = r * r;
    double q = fma(r, hm_b2d(HM_EXP_C5), hm_b2d(HM_EXP_C4));
    q = fma(r, q, hm_b2d(HM_EXP_C3));
    q = fma(r, q, hm_b2d(HM_EXP_C2));
    double p = fma(r2, q, r);
    double y = fma(thi, p, tlo);
    y = thi + y; /* y in [0.997, 2) */
    if (!special)
        return hm_b2d(hm_d2b(y) + ((uint64_t)(int64_t)m << 52));
    if (m > 0) /* may overflow to +inf: one rounding in the last product */
        return (y * hm_b2d((uint64_t)(1023 + m - 1) << 52)) * 2.0;
    /* gradual underflow: exact first scaling, one rounding in the second */
    return (y * hm_b2d((uint64_t)(1023 + m + 600) << 52)) * 0x1p-600;
}

HM_FN double hm_exp_t(double x, const uint64_t *etab) { return hm_exp_dd_t(x, 0.0, etab); }

/* x**y for x >= 0 (Fortran real**real), log carried in double-double. */
HM_FN double hm_pow_t(double x, double y, const uint64_t *ltab, const uint64_t *etab)
{
    double lh, ll;
    hm_log_dd_t(x, ltab, &lh, &ll);
    double eh = y * lh;
    double el = fma(y, lh, -eh) + y * ll;
    return hm_exp_dd_t(eh, el, etab);
}

/* ======================================================================
 * Integer-pipe variants.  On GB300 the FP64 pipe issues ~0.5 T thread-ops/s
 * while the integer pipes are tens of times faster, so the same table-driven
 * reductions are evaluated in 64/128-bit fixed point: log(x) as a Q116
 * number (k*ln2 + logc exact to 2^-107, log1p of the exact reduced argument
 * with relative error < 2^-61), exp from a Q64 argument (Taylor expm1 in
 * Q64, 2^(j/128) in Q63), and one final round-to-nearest-even to double.
 * No FP64 instruction is used on the main paths.  Accuracy (tests/
 * test_hmath.py): < 0.51 ulp for log and exp, < 0.6 ulp for pow.
 * ====================================================================== */
typedef __int128 hm_i128;
typedef unsigned __int128 hm_u128;

static const uint64_t hm_fxlog_tab_h[3 * HM_LOG_N] = HM_FX_LOG_TABLE_INIT;
static const uint64_t hm_fxexp_tab_h[128] = HM_FX_EXP_TABLE_INIT;
#if defined(__CUDACC__)
static __device__ const uint64_t hm_fxlog_tab_d[3 * HM_LOG_N] = HM_FX_LOG_TABLE_INIT;
static __device__ const uint64_t hm_fxexp_tab_d[128] = HM_FX_EXP_TABLE_INIT;
#endif
#if defined(__CUDA_ARCH__)
#define HM_FXLOG_TAB hm_fxlog_tab_d
#define HM_FXEXP_TAB hm_fxexp_tab_d
#else
#define HM_FXLOG_TAB hm_fxlog_tab_h
#define HM_FXEXP_TAB hm_fxexp_tab_h
#endif

HM_FN uint64_t hm_umulhi(uint64_t a, uint64_t b)
{
#if defined(__CUDA_ARCH__)
    return __umul64hi(a, b);
#else
    return (uint64_t)(((hm_u128)a * b) >> 64);
#endif
}

/* floor(a * b / 2^64) for signed a, b */
HM_FN int64_t hm_smulhi(int64_t a, int64_t b)
{
#if defined(__CUDA_ARCH__)
    return __mul64hi(a, b);
#else
    return (int64_t)(((hm_i128)a * b) >> 64);
#endif
}

HM_FN int hm_clz64(uint64_t x) /* x != 0 */
{
#if defined(__CUDA_ARCH__)
    return __clzll((long long)x);
#else
    return __builtin_clzll(x);
#endif
}

HM_FN int hm_clz128(hm_u128 x) /* x != 0 */
{
    uint64_t hi = (uint64_t)(x >> 64);
    return hi ? hm_clz64(hi) : 64 + hm_clz64((uint64_t)x);
}

/* Round mant * 2^(e - 63) (mant in [2^63, 2^64), `sticky` = nonzero bits
 * below mant) to the nearest double, ties to even; gradual underflow and
 * overflow to infinity. */
HM_FN double hm_make_double(int neg, uint64_t mant, int e, int sticky)
{
    const uint64_t sign = neg ? 0x8000000000000000ULL : 0;
    int be = e + 1023;
    if (be >= 2047)
        return hm_b2d(sign | 0x7ff0000000000000ULL);
    int sh = 11;
    if (be <= 0) {
        sh = 11 + 1 - be;
        be = 0;
        if (sh > 64)
            return hm_b2d(sign); /* below half the smallest subnormal */
    }
    uint64_t m53, rem, half;
    if (sh == 64) {
        m53 = 0;
        rem = mant;
        half = 0x8000000000000000ULL;
    } else {
        m53 = mant >> sh;
        rem = mant & ((1ULL << sh) - 1);
        half = 1ULL << (sh - 1);
    }
    if (rem > half || (rem == half && (sticky || (m53 & 1))))
        m53++;
    const uint64_t bits = (be > 0 ? ((uint64_t)(be - 1) << 52) : 0) + m53;
    return hm_b2d(sign | bits);
}

/* log(x) for positive normal-or-subnormal finite x as a Q116 fixed-point
 * number; also returns log1p of the reduced argument as a floating value
 * (neg, mant, e) and whether x lies in the two intervals around 1 where
 * log(x) == log1p(r) (near1).  Caller handles zero / negative / inf / NaN. */
HM_FN hm_i128 hm_log_fx(uint64_t u, int *near1, int *tneg, uint64_t *tmant, int *te)
{
    int64_t kadj = 0;
    if ((u >> 52) == 0) {
        /* subnormal u * 2^-1074: shift the leading 1 to bit 52, which reads
         * as the normal number (u << lz) * 2^-1074 = x * 2^lz */
        const int lz = hm_clz64(u) - 11;
        u <<= lz;
        kadj = -lz;
    }
    const uint64_t tmp = u - HM_LOG_OFF;
    const int64_t k = ((int64_t)tmp >> 52) + kadj;
    const uint32_t i = (uint32_t)(tmp >> (52 - HM_LOG_NBITS)) & (HM_LOG_N - 1);
    const uint64_t iz = u - (tmp & 0xfff0000000000000ULL);
    const uint64_t M = (iz & 0x000fffffffffffffULL) | 0x0010000000000000ULL;
    const uint64_t A = HM_FXLOG_TAB[3 * i];
    const int64_t R = (int64_t)(M * A) - ((int64_t)1 << 61); /* r = z*invc - 1 = R * 2^-61, exact */
    const hm_i128 logc = (hm_i128)(((hm_u128)HM_FXLOG_TAB[3 * i + 1] << 64) | HM_FXLOG_TAB[3 * i + 2]);
    *near1 = (k == 0) && (logc == 0);
    if (R == 0) {
        *tmant = 0;
        return (hm_i128)k * (hm_i128)(((hm_u128)HM_FX_LN2_Q116_HI << 64) | HM_FX_LN2_Q116_LO) + logc;
    }
    /* log1p(r) = r * (1 + r * q(r)), q in Q63, r in Q64 */
    const int64_t rq = R * 8;
    int64_t q = HM_FX_LOG_C7;
    q = HM_FX_LOG_C6 + hm_smulhi(rq, q);
    q = HM_FX_LOG_C5 + hm_smulhi(rq, q);
    q = HM_FX_LOG_C4 + hm_smulhi(rq, q);
    q = HM_FX_LOG_C3 + hm_smulhi(rq, q);
    q = HM_FX_LOG_C2 + hm_smulhi(rq, q);
    const int64_t rqq = hm_smulhi(rq, q);                        /* r*q(r), Q63 */
    const uint64_t f = (uint64_t)(((int64_t)1 << 62) + (rqq >> 1)); /* 1 + r*q(r), Q62 */
    const uint64_t aR = (uint64_t)(R < 0 ? -R : R);
    const int lz = hm_clz64(aR);
    uint64_t mant = hm_umulhi(aR << lz, f);
    const int lz2 = hm_clz64(mant);
    mant <<= lz2;
    const int e = 4 - lz - lz2; /* |log1p(r)| = mant * 2^(e - 63) */
    *tneg = R < 0;
    *tmant = mant;
    *te = e;
    /* S = k*ln2 + logc + log1p(r) in Q116 */
    const int sh = e + 53;
    hm_i128 tau = sh >= 0 ? (hm_i128)((hm_u128)mant << sh) : (hm_i128)(mant >> (-sh < 64 ? -sh : 63));
    if (R < 0)
        tau = -tau;
    return (hm_i128)k * (hm_i128)(((hm_u128)HM_FX_LN2_Q116_HI << 64) | HM_FX_LN2_Q116_LO) + logc + tau;
}

/* Q116 -> nearest double */
HM_FN double hm_q116_to_double(hm_i128 S)
{
    if (S == 0)
        return 0.0;
    const int neg = S < 0;
    const hm_u128 a = (hm_u128)(neg ? -S : S);
    const int lz = hm_clz128(a);
    const hm_u128 n = a << lz;
    return hm_make_double(neg, (uint64_t)(n >> 64), 11 - lz, (uint64_t)n != 0);
}

HM_FN_BIG double hm_log_i(double x)
{
    const uint64_t u = hm_d2b(x);
    const uint32_t top = (uint32_t)(u >> 32);
    if (top >= 0x7ff00000u) { /* +inf, NaN, or negative (sign bit set) */
        if (u == 0x7ff0000000000000ULL)
            return x;
        if (hm_abs_bits(u) == 0)
            return -HUGE_VAL; /* -0 */
        return hm_b2d(0x7ff8000000000000ULL);
    }
    if (u == 0)
        return -HUGE_VAL;
    int near1, tneg, te;
    uint64_t tmant;
    const hm_i128 S = hm_log_fx(u, &near1, &tneg, &tmant, &te);
    if (near1)
        return tmant ? hm_make_double(tneg, tmant, te, 0) : 0.0;
    return hm_q116_to_double(S);
}

/* exp(X * 2^-64) for a signed Q64 argument */
HM_FN_BIG double hm_exp_q64(hm_i128 X)
{
    if (X > ((hm_i128)710 << 64))
        return HUGE_VAL;
    if (X < -((hm_i128)746 << 64))
        return 0.0;
    const int64_t t = (int64_t)(X >> 12);                     /* Q52 */
    const int64_t kq = hm_smulhi(t, (int64_t)HM_FX_INVLN2N_Q54); /* x*128/ln2 in Q42 */
    const int64_t k = (kq + ((int64_t)1 << 41)) >> 42;
    const hm_i128 ln2n = (hm_i128)(((hm_u128)HM_FX_LN2N_Q116_HI << 64) | HM_FX_LN2N_Q116_LO);
    const int64_t r = (int64_t)(X - (((hm_i128)k * ln2n) >> 52)); /* Q64, |r| < 2^-7 */
    int64_t q = HM_FX_EXP_C6;
    q = HM_FX_EXP_C5 + hm_smulhi(r, q);
    q = HM_FX_EXP_C4 + hm_smulhi(r, q);
    q = HM_FX_EXP_C3 + hm_smulhi(r, q);
    q = HM_FX_EXP_C2 + hm_smulhi(r, q);                       /* Q63 */
    const int64_t r2 = hm_smulhi(r, r);                       /* Q64 */
    const int64_t p = r + hm_smulhi(r2, q) * 2;               /* expm1(r), Q64 */
    const uint64_t T = HM_FXEXP_TAB[(uint32_t)k & 127u];      /* 2^(j/128), Q63 */
    const uint64_t tp = hm_umulhi(T, (uint64_t)(p < 0 ? -p : p));
    uint64_t y = p < 0 ? T - tp : T + tp;                     /* Q63 */
    int e = (int)(k >> 7);
    if (!(y >> 63)) {
        y <<= 1;
        e -= 1;
    }
    return hm_make_double(0, y, e, 0);
}

HM_FN double hm_exp_i(double x)
{
    const uint64_t u = hm_d2b(x);
    const uint64_t a = hm_abs_bits(u);
    if (a >= 0x4087500000000000ULL) { /* |x| >= 746, inf or NaN */
        if (a > 0x7ff0000000000000ULL)
            return x;
        return (u >> 63) ? 0.0 : HUGE_VAL;
    }
    const int e = (int)(a >> 52) - 1023;
    const uint64_t M = (a & 0x000fffffffffffffULL) | (a >> 52 ? 0x0010000000000000ULL : 0);
    hm_i128 X;
    if (e + 12 >= 0)
        X = (hm_i128)((hm_u128)M << (e + 12));
    else
        X = (hm_i128)(e + 12 > -64 ? (M >> (-(e + 12))) : 0);
    return hm_exp_q64((u >> 63) ? -X : X);
}

/* x**y for x >= 0 (Fortran real**real): exp(y * log(x)) with log kept in
 * fixed point (no rounding of the intermediate). */
HM_FN_BIG double hm_pow_i(double x, double y)
{
    const uint64_t u = hm_d2b(x);
    const uint64_t uy = hm_d2b(y);
    const uint64_t ay = hm_abs_bits(uy);
    if (ay == 0 || u == 0x3ff0000000000000ULL)
        return 1.0;
    const int ey = (int)(ay >> 52) - 1023;
    if (u - 1 >= 0x7fefffffffffffffULL || ey > 40) {
        /* x zero, negative, inf or NaN, or |y| >= 2^41 (inf/NaN included):
         * the exp(y * log(x)) definition in FP64 */
        return hm_exp_t(y * hm_log_t(x, HM_LOG_TAB), HM_EXP_TAB);
    }
    int near1, tneg, te;
    uint64_t tmant;
    const hm_i128 S = hm_log_fx(u, &near1, &tneg, &tmant, &te) >> 52; /* Q64, |S| < 2^74 */
    const uint64_t My = (ay & 0x000fffffffffffffULL) | (ay >> 52 ? 0x0010000000000000ULL : 0);
    const int neg = (S < 0) != (int)(uy >> 63);
    const hm_u128 aS = (hm_u128)(S < 0 ? -S : S);
    /* aS * My < 2^74 * 2^53: fits in 127 bits */
    const hm_u128 prod = ((hm_u128)((uint64_t)(aS >> 64) * My) << 64) +
                         (((hm_u128)hm_umulhi((uint64_t)aS, My) << 64) | (uint64_t)((uint64_t)aS * My));
    const int sh = 52 - ey; /* >= 12 */
    const hm_i128 P = (hm_i128)(sh < 127 ? prod >> sh : 0);
    return hm_exp_q64(neg ? -P : P);
}

/* ---- the same fixed-point algorithms on explicit 64-bit limbs ----
 * Identical integers (and results) as hm_log_i / hm_exp_i / hm_pow_i above,
 * with fewer instructions: products of a small integer by a 128-bit
 * constant as two 64-bit products, shifts of 64-bit values into 128 bits,
 * and differences known to be small taken modulo 2^64. */

/* (hi, lo) = k * (chi, clo) for |k| < 2^32, as a signed 128-bit value */
HM_FN void hm_mulk128(int64_t k, uint64_t chi, uint64_t clo, int64_t *rhi, uint64_t *rlo)
{
    const uint64_t ak = (uint64_t)(k < 0 ? -k : k);
    uint64_t lo = ak * clo;
    uint64_t hi = ak * chi + hm_umulhi(ak, clo);
    if (k < 0) {
        hi = ~hi + (lo == 0);
        lo = (uint64_t)0 - lo;
    }
    *rhi = (int64_t)hi;
    *rlo = lo;
}

HM_FN void hm_add128(int64_t *hi, uint64_t *lo, int64_t bhi, uint64_t blo)
{
    const uint64_t l = *lo + blo;
    *hi = (int64_t)((uint64_t)*hi + (uint64_t)bhi + (l < blo));
    *lo = l;
}

/* log(x) in Q116 as (hi, lo) limbs; same contract as hm_log_fx */
HM_FN void hm_log_fx2(uint64_t u, int64_t *Shi, uint64_t *Slo, int *near1, int *tneg, uint64_t *tmant, int *te)
{
    int64_t kadj = 0;
    if ((u >> 52) == 0) {
        const int lz = hm_clz64(u) - 11;
        u <<= lz;
        kadj = -lz;
    }
    const uint64_t tmp = u - HM_LOG_OFF;
    const int64_t k = ((int64_t)tmp >> 52) + kadj;
    const uint32_t i = (uint32_t)(tmp >> (52 - HM_LOG_NBITS)) & (HM_LOG_N - 1);
    const uint64_t iz = u - (tmp & 0xfff0000000000000ULL);
    const uint64_t M = (iz & 0x000fffffffffffffULL) | 0x0010000000000000ULL;
    const uint64_t A = HM_FXLOG_TAB[3 * i];
    const int64_t R = (int64_t)(M * A) - ((int64_t)1 << 61);
    const int64_t lchi = (int64_t)HM_FXLOG_TAB[3 * i + 1];
    const uint64_t lclo = HM_FXLOG_TAB[3 * i + 2];
    int64_t hi;
    uint64_t lo;
    hm_mulk128(k, HM_FX_LN2_Q116_HI, HM_FX_LN2_Q116_LO, &hi, &lo);
    hm_add128(&hi, &lo, lchi, lclo);
    *near1 = (k == 0) && (lchi == 0) && (lclo == 0);
    *tmant = 0;
    if (R != 0) {
        const int64_t rq = R * 8;
        int64_t q = HM_FX_LOG_C7;
        q = HM_FX_LOG_C6 + hm_smulhi(rq, q);
        q = HM_FX_LOG_C5 + hm_smulhi(rq, q);
        q = HM_FX_LOG_C4 + hm_smulhi(rq, q);
        q = HM_FX_LOG_C3 + hm_smulhi(rq, q);
        q = HM_FX_LOG_C2 + hm_smulhi(rq, q);
        const int64_t rqq = hm_smulhi(rq, q);
        const uint64_t f = (uint64_t)(((int64_t)1 << 62) + (rqq >> 1));
        const uint64_t aR = (uint64_t)(R < 0 ? -R : R);
        const int lz = hm_clz64(aR);
        uint64_t mant = hm_umulhi(aR << lz, f);
        const int lz2 = hm_clz64(mant);
        mant <<= lz2;
        const int e = 4 - lz - lz2;
        *tneg = R < 0;
        *tmant = mant;
        *te = e;
        const int sh = e + 53; /* <= 46 */
        int64_t thi;
        uint64_t tlo;
        if (sh >= 0) {
            thi = (int64_t)(sh ? mant >> (64 - sh) : 0);
            tlo = mant << sh;
        } else {
            thi = 0;
            tlo = mant >> (-sh < 64 ? -sh : 63);
        }
        if (R < 0) {
            thi = (int64_t)(~(uint64_t)thi + (tlo == 0));
            tlo = (uint64_t)0 - tlo;
        }
        hm_add128(&hi, &lo, thi, tlo);
    }
    *Shi = hi;
    *Slo = lo;
}

HM_FN double hm_q116_to_double2(int64_t hi, uint64_t lo)
{
    if (hi == 0 && lo == 0)
        return 0.0;
    const int neg = hi < 0;
    uint64_t h = (uint64_t)hi, l = lo;
    if (neg) {
        h = ~h + (l == 0);
        l = (uint64_t)0 - l;
    }
    if (h) {
        const int lz = hm_clz64(h);
        const uint64_t top = lz ? (h << lz) | (l >> (64 - lz)) : h;
        const uint64_t rest = l << lz;
        return hm_make_double(neg, top, 11 - lz, rest != 0);
    }
    const int lz = hm_clz64(l);
    return hm_make_double(neg, l << lz, 11 - 64 - lz, 0);
}

HM_FN_BIG double hm_log_i2(double x)
{
    const uint64_t u = hm_d2b(x);
    const uint32_t top = (uint32_t)(u >> 32);
    if (top >= 0x7ff00000u) {
        if (u == 0x7ff0000000000000ULL)
            return x;
        if (hm_abs_bits(u) == 0)
            return -HUGE_VAL;
        return hm_b2d(0x7ff8000000000000ULL);
    }
    if (u == 0)
        return -HUGE_VAL;
    int near1, tneg, te;
    uint64_t tmant;
    int64_t hi;
    uint64_t lo;
    hm_log_fx2(u, &hi, &lo, &near1, &tneg, &tmant, &te);
    if (near1)
        return tmant ? hm_make_double(tneg, tmant, te, 0) : 0.0;
    return hm_q116_to_double2(hi, lo);
}

/* exp of a Q64 argument given as (Xhi, Xlo) limbs (signed 128) */
HM_FN_BIG double hm_exp_q64_2(int64_t Xhi, uint64_t Xlo)
{
    if (Xhi > 710 || (Xhi == 710 && Xlo > 0))
        return HUGE_VAL;
    if (Xhi < -746)
        return 0.0;
    const int64_t t = (int64_t)(((uint64_t)Xhi << 52) | (Xlo >> 12)); /* Q52 */
    const int64_t kq = hm_smulhi(t, (int64_t)HM_FX_INVLN2N_Q54);
    const int64_t k = (kq + ((int64_t)1 << 41)) >> 42;
    int64_t phi;
    uint64_t plo;
    hm_mulk128(k, HM_FX_LN2N_Q116_HI, HM_FX_LN2N_Q116_LO, &phi, &plo);
    const int64_t r = (int64_t)(Xlo - (((uint64_t)phi << 12) | (plo >> 52))); /* Q64, exact mod 2^64 */
    int64_t q = HM_FX_EXP_C6;
    q = HM_FX_EXP_C5 + hm_smulhi(r, q);
    q = HM_FX_EXP_C4 + hm_smulhi(r, q);
    q = HM_FX_EXP_C3 + hm_smulhi(r, q);
    q = HM_FX_EXP_C2 + hm_smulhi(r, q);
    const int64_t r2 = hm_smulhi(r, r);
    const int64_t p = r + hm_smulhi(r2, q) * 2;
    const uint64_t T = HM_FXEXP_TAB[(uint32_t)k & 127u];
    const uint64_t tp = hm_umulhi(T, (uint64_t)(p < 0 ? -p : p));
    uint64_t y = p < 0 ? T - tp : T + tp;
    int e = (int)(k >> 7);
    if (!(y >> 63)) {
        y <<= 1;
        e -= 1;
    }
    return hm_make_double(0, y, e, 0);
}

HM_FN double hm_exp_i2(double x)
{
    const uint64_t u = hm_d2b(x);
    const uint64_t a = hm_abs_bits(u);
    if (a >= 0x4087500000000000ULL) {
        if (a > 0x7ff0000000000000ULL)
            return x;
        return (u >> 63) ? 0.0 : HUGE_VAL;
    }
    const int e = (int)(a >> 52) - 1023;
    const uint64_t M = (a & 0x000fffffffffffffULL) | (a >> 52 ? 0x0010000000000000ULL : 0);
    const int s = e + 12; /* X = M * 2^s, s <= 21 */
    uint64_t hi, lo;
    if (s >= 0) {
        hi = s ? M >> (64 - s) : 0;
        lo = M << s;
    } else {
        hi = 0;
        lo = s > -64 ? M >> (-s) : 0;
    }
    if (u >> 63) {
        hi = ~hi + (lo == 0);
        lo = (uint64_t)0 - lo;
    }
    return hm_exp_q64_2((int64_t)hi, lo);
}

HM_FN_BIG double hm_pow_i2(double x, double y)
{
    const uint64_t u = hm_d2b(x);
    const uint64_t uy = hm_d2b(y);
    const uint64_t ay = hm_abs_bits(uy);
    if (ay == 0 || u == 0x3ff0000000000000ULL)
        return 1.0;
    const int ey = (int)(ay >> 52) - 1023;
    if (u == 0 && ay < 0x7ff0000000000000ULL) /* +0 ** finite y: exp(y * -inf) */
        return (uy >> 63) ? HUGE_VAL : 0.0;
    if (u - 1 >= 0x7fefffffffffffffULL || ey > 40)
        return hm_exp_t(y * hm_log_t(x, HM_LOG_TAB), HM_EXP_TAB);
    int near1, tneg, te;
    uint64_t tmant;
    int64_t Shi;
    uint64_t Slo;
    hm_log_fx2(u, &Shi, &Slo, &near1, &tneg, &tmant, &te);
    /* S >> 52 (Q64), |S| < 2^74 */
    int64_t shi = Shi >> 52;
    uint64_t slo = ((uint64_t)Shi << 12) | (Slo >> 52);
    const uint64_t My = (ay & 0x000fffffffffffffULL) | (ay >> 52 ? 0x0010000000000000ULL : 0);
    const int neg = (shi < 0) != (int)(uy >> 63);
    uint64_t ahi = (uint64_t)shi, alo = slo;
    if (shi < 0) {
        ahi = ~ahi + (alo == 0);
        alo = (uint64_t)0 - alo;
    }
    /* prod = |S| * My < 2^127 */
    const uint64_t plo = alo * My;
    const uint64_t phi = ahi * My + hm_umulhi(alo, My);
    const int sh = 52 - ey; /* >= 12 */
    uint64_t rhi, rlo;
    if (sh < 64) {
        rlo = (plo >> sh) | (phi << (64 - sh));
        rhi = phi >> sh;
    } else if (sh < 128) {
        rlo = phi >> (sh - 64);
        rhi = 0;
    } else {
        rlo = 0;
        rhi = 0;
    }
    if (neg) {
        rhi = ~rhi + (rlo == 0);
        rlo = (uint64_t)0 - rlo;
    }
    return hm_exp_q64_2((int64_t)rhi, rlo);
}

/* log10(x) = log(x) / ln 10 from the fixed-point logarithm, one rounding */
HM_FN_BIG double hm_log10_i2(double x)
{
    const uint64_t u = hm_d2b(x);
    const uint32_t top = (uint32_t)(u >> 32);
    if (top >= 0x7ff00000u || u == 0)
        return hm_log_i2(x); /* +-0, negative, inf, NaN: same special values */
    int near1, tneg, te;
    uint64_t tmant;
    int64_t hi;
    uint64_t lo;
    hm_log_fx2(u, &hi, &lo, &near1, &tneg, &tmant, &te);
    const uint64_t c = HM_FX_INVLN10_Q64;
    if (near1) { /* log(x) = log1p(r), a floating value (tneg, tmant, te) */
        if (!tmant)
            return 0.0;
        uint64_t m = hm_umulhi(tmant, c); /* mant * c / 2^64 */
        int e = te;
        const int lz = hm_clz64(m);
        m <<= lz;
        e -= lz;
        return hm_make_double(tneg, m, e, 0);
    }
    const int neg = hi < 0;
    uint64_t ah = (uint64_t)hi, al = lo;
    if (neg) {
        ah = ~ah + (al == 0);
        al = (uint64_t)0 - al;
    }
    /* (|S| * c) >> 64 in Q116 */
    uint64_t rlo = ah * c;
    uint64_t rhi = hm_umulhi(ah, c);
    const uint64_t add = hm_umulhi(al, c);
    rlo += add;
    rhi += (rlo < add);
    if (neg) {
        rhi = ~rhi + (rlo == 0);
        rlo = (uint64_t)0 - rlo;
    }
    return hm_q116_to_double2((int64_t)rhi, rlo);
}

#ifndef HM_FP64_MATH
HM_FN double hm_log10(double x) { return hm_log10_i2(x); }
HM_FN double hm_log(double x) { return hm_log_i2(x); }
HM_FN double hm_exp(double x) { return hm_exp_i2(x); }
HM_FN double hm_pow(double x, double y) { return hm_pow_i2(x, y); }
#else
HM_FN double hm_log(double x) { return hm_log_t(x, HM_LOG_TAB); }
HM_FN double hm_exp(double x) { return hm_exp_t(x, HM_EXP_TAB); }
HM_FN double hm_pow(double x, double y) { return hm_pow_t(x, y, HM_LOG_TAB, HM_EXP_TAB); }
HM_FN double hm_log10(double x) { return hm_log_t(x, HM_LOG_TAB) / 2.302585092994045684; }
#endif

#endif /* MHM_HMATH_H */
