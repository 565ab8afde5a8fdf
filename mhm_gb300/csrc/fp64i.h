/*
 * fp64i.h -- IEEE-754 double comparisons and division on the integer pipe.
 *
 * GB300's FP64 pipe issues ~0.5 T thread-ops/s, and a double compare (DSETP)
 * or the refinement steps of a double division occupy it like an FMA; the
 * integer pipes are tens of times faster.  Sign masks on a double's bits go
 * through hm_abs_bits, or the compiler turns them back into FP64 |x|.  These functions return exactly
 * what the IEEE operations return (round-to-nearest-even), so kernels that
 * use them stay bit-identical to host code using plain C operators.
 *
 * Comparisons: hm_gt/ge/lt/le follow IEEE for all non-NaN operands (+0 == -0,
 * infinities ordered); the *_ieee variants are also false for NaN operands.
 * Division: hm_div(a, b) == a / b for all inputs; normal/zero operands with a
 * normal result take the integer path (float reciprocal seed, two Newton
 * steps in 64-bit fixed point, exact remainder correction, RNE); everything
 * else (subnormal, infinite, NaN, zero divisor, out-of-range results) uses
 * the native division.  hm_div_r(a, b, hm_recip_of(b)) is the same division
 * with the divisor's reciprocal computed beforehand.
 */
#ifndef MHM_FP64I_H
#define MHM_FP64I_H

#include "hmath.h"

/* order key: monotone in the value for non-NaN doubles, +0 and -0 -> 0
 * (the sign-cleared bits through hm_abs_bits, which stays on the integer
 * pipe) */
HM_FN int64_t hm_okey(double x)
{
    const uint64_t u = hm_d2b(x);
    const int64_t m = (int64_t)hm_abs_bits(u);
    return (int64_t)u < 0 ? -m : m;
}
HM_FN int hm_isnan_i(double x) { return hm_abs_bits(hm_d2b(x)) > 0x7ff0000000000000ULL; }
HM_FN int hm_gt(double a, double b) { return hm_okey(a) > hm_okey(b); }
HM_FN int hm_ge(double a, double b) { return hm_okey(a) >= hm_okey(b); }
HM_FN int hm_lt(double a, double b) { return hm_okey(a) < hm_okey(b); }
HM_FN int hm_le(double a, double b) { return hm_okey(a) <= hm_okey(b); }
HM_FN int hm_gt_ieee(double a, double b) { return !hm_isnan_i(a) && !hm_isnan_i(b) && hm_gt(a, b); }
HM_FN int hm_lt_ieee(double a, double b) { return !hm_isnan_i(a) && !hm_isnan_i(b) && hm_lt(a, b); }
HM_FN int hm_ge_ieee(double a, double b) { return !hm_isnan_i(a) && !hm_isnan_i(b) && hm_ge(a, b); }
/* x > 0, x < 0 against the constant zero */
HM_FN int hm_gt0(double x) { return hm_okey(x) > 0; }
HM_FN int hm_lt0(double x) { return hm_okey(x) < 0; }
/* c ? a : b as a select of the bit patterns: a select of doubles is issued
 * as an FP64-pipe move on this GPU (measured), an integer select is not */
HM_FN double hm_sel(int c, double a, double b) { return hm_b2d(c ? hm_d2b(a) : hm_d2b(b)); }
/* -x as a flip of the sign bit on the integer pipe (inline PTX on the device,
 * so that it is not turned into an FP64 negation); a + (-b) is exactly a - b */
HM_FN double hm_neg(double x)
{
#if defined(__CUDA_ARCH__)
    uint64_t r;
    asm("xor.b64 %0, %1, 0x8000000000000000;" : "=l"(r) : "l"(hm_d2b(x)));
    return hm_b2d(r);
#else
    return hm_b2d(hm_d2b(x) ^ 0x8000000000000000ULL);
#endif
}
/* min/max with the selection rules of the reference's (a < b ? a : b) */
HM_FN double hm_min_sel(double a, double b) { return hm_sel(hm_lt(a, b), a, b); }

/* reciprocal seed 1/x in float, correctly rounded on host and device */
HM_FN float hm_frcp(float x)
{
#if defined(__CUDA_ARCH__)
    return __frcp_rn(x);
#else
    return 1.0f / x;
#endif
}

HM_FN uint32_t hm_f2b(float f)
{
#if defined(__CUDA_ARCH__)
    return (uint32_t)__float_as_uint(f);
#else
    uint32_t b;
    memcpy(&b, &f, sizeof b);
    return b;
#endif
}

/* 64-bit fixed-point reciprocal of a divisor mantissa Mb in (2^52, 2^53):
 * inv ~ 2^116 / Mb < 2^64 from a float seed (~24 bits) and two Newton steps
 * y' = y (2 - Mb y / 2^116), which approach from below.  Depends on the
 * divisor only, so a divisor that stays fixed over many divisions (a cell's
 * soil parameters over a chunk of steps) needs it once: hm_recip_of. */
HM_FN uint64_t hm_recip_mant(uint64_t Mb)
{
    const float fy = hm_frcp((float)(uint32_t)(Mb >> 29)); /* in (2^-24, 2^-23] */
    const uint32_t fb = hm_f2b(fy);
    const int sh = (int)((fb >> 23) & 0xffu) - 127 - 23 + 116 - 29; /* 40 or 41 */
    const uint64_t fm = (uint64_t)((fb & 0x7fffffu) | 0x800000u);
    uint64_t inv = (sh >= 41 && fm == 0x800000u) ? 0xffffffffffffffffULL : fm << sh;
    for (int it = 0; it < 2; ++it) {
        /* err = (2^116 - Mb*inv) >> 52, |err| < 2^42: bits 52..115 of the
         * 128-bit difference, from its two limbs */
        const uint64_t t_lo = Mb * inv, t_hi = hm_umulhi(Mb, inv);
        const uint64_t e_lo = (uint64_t)0 - t_lo;
        const uint64_t e_hi = ((uint64_t)1 << 52) - t_hi - (t_lo != 0);
        const int64_t err_s = (int64_t)((e_hi << 12) | (e_lo >> 52));
        inv = inv + (uint64_t)(hm_smulhi((int64_t)(inv >> 1), err_s) * 2);
    }
    return inv;
}

/* The reciprocal hm_div_r wants for divisor b (0 when b takes another path:
 * zero, subnormal, infinite, NaN or a power of two). */
HM_FN uint64_t hm_recip_of(double b)
{
    const uint64_t ub = hm_d2b(b);
    const uint32_t ebf = (uint32_t)(ub >> 52) & 0x7ffu;
    const uint64_t Mb = (ub & 0x000fffffffffffffULL) | 0x0010000000000000ULL;
    if (ebf - 1u >= 0x7feu || Mb == 0x0010000000000000ULL) return 0;
    return hm_recip_mant(Mb);
}

/* a / b, correctly rounded, given inv = hm_recip_of(b) */
HM_FN_BIG double hm_div_r(double a, double b, uint64_t inv)
{
    const uint64_t ua = hm_d2b(a), ub = hm_d2b(b);
    const uint32_t eaf = (uint32_t)(ua >> 52) & 0x7ffu, ebf = (uint32_t)(ub >> 52) & 0x7ffu;
    const uint64_t sign = (ua ^ ub) & 0x8000000000000000ULL;
    if (ebf - 1u >= 0x7feu || (eaf - 1u >= 0x7feu && hm_abs_bits(ua) != 0))
        return a / b; /* b zero/subnormal/inf/NaN, or a subnormal/inf/NaN */
    if (hm_abs_bits(ua) == 0)
        return hm_b2d(sign); /* +-0 / normal */
    uint64_t Ma = (ua & 0x000fffffffffffffULL) | 0x0010000000000000ULL;
    const uint64_t Mb = (ub & 0x000fffffffffffffULL) | 0x0010000000000000ULL;
    int e = (int)eaf - (int)ebf; /* unbiased exponent of the quotient */
    if (Ma < Mb) {
        Ma <<= 1;
        e -= 1;
    }
    if (e > 1023 || e < -1022)
        return a / b; /* overflow or subnormal result: native path */
    uint64_t Q;
    hm_i128 R;
    if (Mb == 0x0010000000000000ULL) { /* b is a power of two: exact */
        Q = Ma << 2;
        R = 0;
    } else {
        /* Q ~ floor(Ma * 2^54 / Mb) in [2^54, 2^55) */
        Q = (hm_umulhi(Ma, inv) << 2) | ((Ma * inv) >> 62);
        /* exact remainder Ma*2^54 - Q*Mb; |R| < 2^57, so modulo 2^64 suffices */
        int64_t r = (int64_t)((Ma << 54) - Q * Mb);
        for (int c = 0; c < 3; ++c) {
            if (r < 0) {
                Q -= 1;
                r += (int64_t)Mb;
            } else if (r >= (int64_t)Mb) {
                Q += 1;
                r -= (int64_t)Mb;
            }
        }
        R = r;
    }
    /* round Q (55 bits: 53 + guard + round) to nearest even */
    uint64_t m53 = Q >> 2;
    const uint32_t g = (uint32_t)(Q & 3u);
    const int sticky = R != 0;
    if (g > 2 || (g == 2 && (sticky || (m53 & 1))))
        m53++;
    /* m53 in [2^52, 2^53]; a carry to 2^53 moves into the exponent field */
    return hm_b2d(sign | (((uint64_t)(e + 1022) << 52) + m53));
}

/* a / b, correctly rounded */
HM_FN_BIG double hm_div(double a, double b) { return hm_div_r(a, b, hm_recip_of(b)); }

#endif /* MHM_FP64I_H */
