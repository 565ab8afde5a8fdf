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
#else
#include <math.h>
#include <string.h>
#define HM_FN static inline
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
        if ((u << 1) == 0) {               /* +-0 */
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

HM_FN double hm_log(double x) { return hm_log_t(x, HM_LOG_TAB); }
HM_FN double hm_exp(double x) { return hm_exp_t(x, HM_EXP_TAB); }
HM_FN double hm_pow(double x, double y) { return hm_pow_t(x, y, HM_LOG_TAB, HM_EXP_TAB); }

#endif /* MHM_HMATH_H */
