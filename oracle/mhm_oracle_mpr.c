/*
 * mhm_oracle_mpr.c -- CPU restatement of mHM's multiscale parameter
 * regionalisation (MPR) for one land-cover scene (TEST INFRASTRUCTURE: the
 * checker for the GPU MPR kernels).  Literal per-L0-cell loops, in the
 * reference's evaluation and summation order.  Citations: mHM src/MPR/.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "mhm_oracle.h"

#ifdef ORACLE_LIBM
#define ORA_EXP(x) exp(x)
#define ORA_LOG(x) log(x)
#define ORA_LOG10(x) log10(x)
#define ORA_POW(x, y) pow((x), (y))
#else
#include "hmath.h"
#define ORA_EXP(x) hm_exp(x)
#define ORA_LOG(x) hm_log(x)
#define ORA_LOG10(x) hm_log10(x)
#define ORA_POW(x, y) hm_pow((x), (y))
#endif

#define NODATA_DP (-9999.0)

/* src/MPR/mo_mpr_constants.f90 */
static const double BULKDENS_ORGMATTER = 0.224, FIELD_CAP_C1 = -0.60, FIELD_CAP_C2 = 2.0;
static const double VG_SANDTRESH = 66.5;
static const double VGN_C1 = 1.392, VGN_C2 = 0.418, VGN_C3 = -0.024, VGN_C4 = 1.212, VGN_C5 = -0.704,
                    VGN_C6 = -0.648, VGN_C7 = 0.023, VGN_C8 = 0.044, VGN_C9 = 3.168, VGN_C10 = -2.562,
                    VGN_C11 = 7.0E-9, VGN_C12 = 4.004, VGN_C13 = 3.750, VGN_C14 = -0.016, VGN_C15 = -4.197,
                    VGN_C16 = 0.013, VGN_C17 = 0.076, VGN_C18 = 0.276;
static const double KS_C = 10.0, PWP_C = 1.0, PWP_MATPOT_THETAR = 15000.0;

/* src/MPR/mo_mpr_soilmoist.f90:736-772 */
void ora_hydro_cond(const double *param, double sand, double clay, double *Ks)
{
    double x = param[0] + param[1] * sand - param[2] * clay;
    *Ks = param[3] * ORA_EXP(x * ORA_LOG(KS_C));
    if (*Ks < 1.10)
        *Ks = 1.10;
}

/* src/MPR/mo_mpr_soilmoist.f90:626-698 (messages dropped) */
void ora_genuchten(const double *param, double sand, double clay, double Db, double *thetaS, double *n,
                   double *alpha)
{
    double x;
    if (sand < VG_SANDTRESH) {
        *thetaS = param[0] + param[1] * clay + param[2] * Db;
        *n = VGN_C1 - VGN_C2 * ORA_POW(sand, VGN_C3) + VGN_C4 * ORA_POW(clay, VGN_C5);
        x = VGN_C6 + VGN_C7 * sand + VGN_C8 * clay - VGN_C9 * Db;
    } else {
        *thetaS = param[3] + param[4] * clay + param[5] * Db;
        *n = VGN_C10 + VGN_C11 * ORA_POW(sand, VGN_C12) + VGN_C13 * ORA_POW(clay, VGN_C14);
        x = VGN_C15 + VGN_C16 * sand + VGN_C17 * clay - VGN_C18 * Db;
    }
    *alpha = ORA_EXP(x);
    if (*thetaS < 0.01)
        *thetaS = 0.01;
    if (*thetaS > 1.0)
        *thetaS = 1.0;
    if (*n < 1.01000)
        *n = 1.01000;
    if (*alpha < 0.00001)
        *alpha = 0.00001;
}

/* src/MPR/mo_mpr_soilmoist.f90:560-584 */
void ora_field_cap(double Ks, double thetaS, double n, double *thetaFC)
{
    double x = (FIELD_CAP_C1) * (FIELD_CAP_C2 + ORA_LOG10(Ks));
    *thetaFC = thetaS * ORA_EXP(x * ORA_LOG(n));
}

/* src/MPR/mo_mpr_soilmoist.f90:489-520 */
void ora_pwp(double n, double alpha, double thetaS, double *thetaPWP)
{
    double m = PWP_C - (PWP_C / n);
    double x = PWP_C + ORA_EXP(n * ORA_LOG(alpha * PWP_MATPOT_THETAR));
    x = ORA_EXP(m * ORA_LOG(x));
    if (x < 1.0)
        x = 1.0;
    *thetaPWP = thetaS / x;
}

/* upscale_arithmetic_mean, src/MPR/mo_upscaling_operators.f90:266-329: masked
 * block sum in column-major order (rows fastest), divided by n_subcells */
static double upscale_arith(const ora_mpr_domain *d, int k1, const double *v0)
{
    double s = 0.0;
    for (int j = d->left1[k1]; j <= d->right1[k1]; ++j)
        for (int i = d->up1[k1]; i <= d->down1[k1]; ++i) {
            int k0 = d->id0_2d[(size_t)(j - 1) * d->nrows0 + (i - 1)];
            if (k0 >= 0)
                s = s + v0[k0];
        }
    return s / (double)d->nsub1[k1];
}

/* upscale_harmonic_mean, :369-432: n / masked sum of 1/x */
static double upscale_harm(const ora_mpr_domain *d, int k1, const double *v0)
{
    double s = 0.0;
    for (int j = d->left1[k1]; j <= d->right1[k1]; ++j)
        for (int i = d->up1[k1]; i <= d->down1[k1]; ++i) {
            int k0 = d->id0_2d[(size_t)(j - 1) * d->nrows0 + (i - 1)];
            if (k0 >= 0)
                s = s + 1.0 / v0[k0];
        }
    return (double)d->nsub1[k1] / s;
}

/* L0_fractionalCover_in_Lx, :152-227 */
static double fraction_cover(const ora_mpr_domain *d, int k1, const int32_t *cls0, int32_t id)
{
    int cnt = 0;
    for (int j = d->left1[k1]; j <= d->right1[k1]; ++j)
        for (int i = d->up1[k1]; i <= d->down1[k1]; ++i) {
            int k0 = d->id0_2d[(size_t)(j - 1) * d->nrows0 + (i - 1)];
            if (k0 >= 0 && cls0[k0] == id)
                cnt++;
        }
    return (double)cnt / (double)d->nsub1[k1];
}

#define IX2(s, j) ((size_t)(s) * d->maxHor + (j))                       /* (soil, horizon) */
#define IX3(s, j, l) (((size_t)(s) * d->maxHor + (j)) * 3 + (l))         /* (soil, horizon, LC) */

int ora_mpr(const ora_mpr_domain *d, const ora_gamma *g, ora_mpr_out *o)
{
    const int N0 = d->nCells0, N1 = d->nCells1, H = d->nH, nS = d->nSoil, mH = d->maxHor;
    const int nLAI = d->nLAI > 0 ? d->nLAI : 12; /* size(LAI0, 2): monthly slots or a gridded series */
    if (H < 2 || d->proc_sm < 1 || d->proc_sm > 4)
        return -1;
    double *KsVar_H0 = (double *)calloc((size_t)N0, sizeof(double));
    double *KsVar_V0 = (double *)calloc((size_t)N0, sizeof(double));
    double *SMs_FC0 = (double *)calloc((size_t)N0, sizeof(double));
    double *tmp0 = (double *)calloc((size_t)N0, sizeof(double));
    double *t1 = (double *)calloc((size_t)N0, sizeof(double));
    double *t2 = (double *)calloc((size_t)N0, sizeof(double));
    double *t3 = (double *)calloc((size_t)N0, sizeof(double));
    double *t4 = (double *)calloc((size_t)N0, sizeof(double));
    double *t5 = (double *)calloc((size_t)N0, sizeof(double));
    double *Ks = (double *)calloc((size_t)nS * mH * 3, sizeof(double));
    double *Db = (double *)calloc((size_t)nS * mH * 3, sizeof(double));
    double *thS_t = (double *)calloc((size_t)nS * mH * 3, sizeof(double));
    double *thFC_t = (double *)calloc((size_t)nS * mH * 3, sizeof(double));
    double *thPW_t = (double *)calloc((size_t)nS * mH * 3, sizeof(double));
    double *thS = (double *)calloc((size_t)nS * mH, sizeof(double));
    double *thFC = (double *)calloc((size_t)nS * mH, sizeof(double));
    double *thPW = (double *)calloc((size_t)nS * mH, sizeof(double));
    double *fForest = (double *)calloc((size_t)N1, sizeof(double));
    double *fPerm = (double *)calloc((size_t)N1, sizeof(double));
    int rc = 0;
    if (!KsVar_H0 || !KsVar_V0 || !SMs_FC0 || !tmp0 || !t1 || !t2 || !t3 || !t4 || !t5 || !Ks || !Db || !thS_t ||
        !thFC_t || !thPW_t || !thS || !thFC || !thPW || !fForest || !fPerm) {
        rc = -2;
        goto done;
    }
    /* ---- land cover fractions and snow (mo_multi_param_reg.f90:273-320, 800-852) ---- */
    for (int k = 0; k < N1; ++k) {
        fForest[k] = fraction_cover(d, k, d->LCover0, 1);
        o->fSealed[k] = fraction_cover(d, k, d->LCover0, 2);
        fPerm[k] = fraction_cover(d, k, d->LCover0, 3);
        o->fSealed[k] = d->fracSealed_cityArea * o->fSealed[k];
        fPerm[k] = 1.0 - o->fSealed[k] - fForest[k];
        const double *p = g->snow;
        double ddf_f = p[1], ddf_i = p[1] + p[3] + p[2], ddf_p = p[1] + p[3];
        double mdf_f = p[1] + p[5], mdf_i = p[1] + p[3] + p[2] + p[6], mdf_p = p[1] + p[3] + p[7];
        o->tempThresh[k] = p[0];
        o->degDayInc[k] = p[4];
        o->degDayNoPre[k] = (ddf_f * fForest[k] + ddf_i * o->fSealed[k] + ddf_p * fPerm[k]);
        o->degDayMax[k] = (mdf_f * fForest[k] + mdf_i * o->fSealed[k] + mdf_p * fPerm[k]);
    }
    /* ---- mpr_sm, src/MPR/mo_mpr_soilmoist.f90:100-455 (iFlag_soilDB = 0) ---- */
    {
        const double *param = g->soil;
        double om_forest = (d->proc_sm <= 2) ? param[2] + param[0] : param[0];
        double om_imp = param[1], om_perv = param[2];
        int min_nTH = 1 << 30, maxLC = 0;
        for (int s = 0; s < nS; ++s)
            if (d->nTill[s] < min_nTH)
                min_nTH = d->nTill[s];
        for (int k = 0; k < N0; ++k)
            if (d->LCover0[k] > maxLC)
                maxLC = d->LCover0[k];
        for (int s = 0; s < nS; ++s) {
            if (!d->present[s])
                continue;
            for (int j = 0; j < d->nHor[s]; ++j) {
                double Ks_tmp, n, alpha;
                ora_hydro_cond(param + 9, d->sand[IX2(s, j)], d->clay[IX2(s, j)], &Ks_tmp);
                for (int l = 0; l < 3; ++l)
                    Ks[IX3(s, j, l)] = Ks_tmp;
                if (j + 1 <= d->nTill[s]) {
                    for (int L = 1; L <= maxLC; ++L) {
                        double pOM = (L == 1) ? om_forest : (L == 2) ? om_imp : om_perv;
                        double pM = 100.0 - pOM;
                        size_t ix = IX3(s, j, L - 1);
                        Db[ix] = 100.0 / ((pOM / BULKDENS_ORGMATTER) + (pM / d->DbM[IX2(s, j)]));
                        Ks[ix] = Ks[ix] * (d->DbM[IX2(s, j)] / Db[ix]);
                        ora_genuchten(param + 3, d->sand[IX2(s, j)], d->clay[IX2(s, j)], Db[ix], &thS_t[ix], &n, &alpha);
                        ora_field_cap(Ks[ix], thS_t[ix], n, &thFC_t[ix]);
                        ora_pwp(n, alpha, thS_t[ix], &thPW_t[ix]);
                    }
                } else {
                    size_t ix = IX2(s, j + 1 - min_nTH - 1);
                    ora_genuchten(param + 3, d->sand[IX2(s, j)], d->clay[IX2(s, j)], d->DbM[IX2(s, j)], &thS[ix], &n,
                                  &alpha);
                    ora_field_cap(Ks[IX3(s, j, 0)], thS[ix], n, &thFC[ix]);
                    ora_pwp(n, alpha, thS[ix], &thPW[ix]);
                }
            }
        }
        for (int k = 0; k < N0; ++k) {
            int s = d->soilId0[k] - 1, l = d->LCover0[k] - 1;
            double kh = 0.0, kv = 0.0, fc = 0.0, tot = 0.0;
            for (int j = 0; j < d->nHor[s]; ++j) {
                if (j + 1 <= d->nTill[s]) {
                    size_t ix = IX3(s, j, l);
                    kh = kh + thS_t[ix] * Ks[ix];
                    kv = kv + thS_t[ix] / Ks[ix];
                    fc = fc + thFC_t[ix];
                    tot = tot + thS_t[ix];
                } else {
                    size_t ix = IX2(s, j + 1 - min_nTH - 1);
                    kh = kh + thS[ix] * Ks[IX3(s, j, 0)];
                    kv = kv + thS[ix] / Ks[IX3(s, j, 0)];
                    fc = fc + thFC[ix];
                    tot = tot + thS[ix];
                }
            }
            SMs_FC0[k] = (tot - fc) / tot;
            KsVar_H0[k] = kh / tot / param[12];
            KsVar_V0[k] = tot / kv / param[12];
        }
        /* ---- mpr_SMhorizons, src/MPR/mo_mpr_smhorizons.f90:120-741 (iFlag_soilDB = 0) ---- */
        /* the first 13 soil parameters go to mpr_sm, the next 4 (cases 1, 2) or 8
         * (cases 3, 4) to mpr_SMhorizons (mo_multi_param_reg.f90:369-419) */
        const double *p2 = g->soil + 13;
        double rc_forest = p2[0], rc_imp = p2[1], rc_perv = 0, rc_sand = 0, rc_clay = 0, fcmin = 0, fcmax = 0;
        if (d->proc_sm <= 2) {
            rc_perv = p2[0] - p2[2];
        } else {
            rc_perv = p2[2];
            rc_sand = p2[5] - p2[4];
            rc_clay = p2[5];
            fcmin = p2[6];
            fcmax = p2[6] + p2[7];
        }
        for (int h = 0; h < H; ++h) {
            double dpth_f = 0.0, dpth_t = d->horizonDepth[h];
            if (h > 0 && h < H - 1) {
                dpth_f = d->horizonDepth[h - 1];
                dpth_t = d->horizonDepth[h];
            }
            double *Bd0 = t1, *SMs0 = t2, *FC0 = t3, *PW0 = t4, *fR0 = t5;
            for (int k = 0; k < N0; ++k) {
                int l = d->LCover0[k] - 1, s = d->soilId0[k] - 1, nT = d->nTill[s], nHs = d->nHor[s];
                const double *wd = d->Wd + ((size_t)s * H + h) * mH;
                double a = 0.0, b = 0.0;
                for (int j = 0; j < nT; ++j)
                    if (wd[j] > 0.0)
                        a = a + Db[IX3(s, j, l)] * wd[j];
                for (int j = nT; j < nHs; ++j)
                    if (wd[j] >= 0.0)
                        b = b + d->DbM[IX2(s, j)] * wd[j];
                Bd0[k] = a + b;
                a = 0.0;
                b = 0.0;
                for (int j = 0; j < nT; ++j)
                    if (wd[j] > 0.0)
                        a = a + thS_t[IX3(s, j, l)] * wd[j];
                for (int j = nT; j < nHs; ++j)
                    if (wd[j] > 0.0)
                        b = b + thS[IX2(s, j + 1 - min_nTH - 1)] * wd[j];
                SMs0[k] = a + b;
                a = 0.0;
                b = 0.0;
                for (int j = 0; j < nT; ++j)
                    if (wd[j] > 0.0)
                        a = a + thFC_t[IX3(s, j, l)] * wd[j];
                for (int j = nT; j < nHs; ++j)
                    if (wd[j] > 0.0)
                        b = b + thFC[IX2(s, j + 1 - min_nTH - 1)] * wd[j];
                FC0[k] = a + b;
                a = 0.0;
                b = 0.0;
                for (int j = 0; j < nT; ++j)
                    if (wd[j] > 0.0)
                        a = a + thPW_t[IX3(s, j, l)] * wd[j];
                for (int j = nT; j < nHs; ++j)
                    if (wd[j] > 0.0)
                        b = b + thPW[IX2(s, j + 1 - min_nTH - 1)] * wd[j];
                PW0[k] = a + b;
                if (h == H - 1) {
                    dpth_f = d->horizonDepth[H - 2];
                    dpth_t = d->RZdepth[s];
                }
                SMs0[k] = SMs0[k] * (dpth_t - dpth_f);
                FC0[k] = FC0[k] * (dpth_t - dpth_f);
                PW0[k] = PW0[k] * (dpth_t - dpth_f);
            }
            /* root fractions use dpth_f/dpth_t as left by the loop above */
            for (int k = 0; k < N0; ++k) {
                int L = d->LCover0[k];
                double c;
                if (L == 1) {
                    c = rc_forest;
                } else if (L == 2) {
                    c = rc_imp;
                } else if (d->proc_sm <= 2) {
                    c = rc_perv;
                } else {
                    double fcn = (((FC0[k] / (dpth_t - dpth_f)) - fcmin) / (fcmax - fcmin));
                    if (fcn < 0.0)
                        fcn = 0.0;
                    else if (fcn > 1.0)
                        fcn = 1.0;
                    c = (fcn * rc_clay) + ((1 - fcn) * rc_sand);
                }
                fR0[k] = (1.0 - ORA_POW(c, dpth_t * 0.1)) - (1.0 - ORA_POW(c, dpth_f * 0.1));
            }
            for (int k = 0; k < N0; ++k)
                tmp0[k] = Bd0[k] * p2[3]; /* beta0 = Bd0 * param(4) */
            for (int k = 0; k < N1; ++k) {
                size_t o1 = (size_t)h * N1 + k;
                o->SMs[o1] = upscale_harm(d, k, SMs0);
                o->beta[o1] = upscale_harm(d, k, tmp0);
                o->PW[o1] = upscale_harm(d, k, PW0);
                o->FC[o1] = upscale_harm(d, k, FC0);
                o->fRoots[o1] = upscale_harm(d, k, fR0);
            }
        }
        for (int k = 0; k < N1; ++k) {
            for (int h = 0; h < H; ++h) {
                size_t o1 = (size_t)h * N1 + k;
                if (o->FC[o1] > o->SMs[o1])
                    o->FC[o1] = o->SMs[o1] - 0.01 * o->SMs[o1];
                if (o->PW[o1] > o->FC[o1])
                    o->PW[o1] = o->FC[o1] - 0.01 * o->FC[o1];
                if (o->SMs[o1] < 0.0)
                    o->SMs[o1] = 0.0001;
                if (o->FC[o1] < 0.0)
                    o->FC[o1] = 0.0001;
                if (o->PW[o1] < 0.0)
                    o->PW[o1] = 0.0001;
            }
            double tot = 0.0;
            for (int h = 0; h < H; ++h)
                if (o->fRoots[(size_t)h * N1 + k] > 0.0)
                    tot = tot + o->fRoots[(size_t)h * N1 + k];
            for (int h = 0; h < H; ++h)
                o->fRoots[(size_t)h * N1 + k] = (tot > 0.0) ? o->fRoots[(size_t)h * N1 + k] / tot : 0.0;
        }
        for (int k = 0; k < N1; ++k)
            o->jarvis_c1[k] = (d->proc_sm == 2 || d->proc_sm == 3) ? g->soil[d->n_soil_params - 1] : 0.0;
    }
    /* ---- PET correction by LAI, src/MPR/mo_mpr_pet.f90:60-140 (harmonic mean) ---- */
    if (d->proc_pet == -1) {
        const double *p = g->pet;
        for (int m = 0; m < nLAI; ++m) {
            for (int k = 0; k < N0; ++k) {
                int L = d->LCover0[k];
                double base = (L == 1) ? p[0] : (L == 2) ? p[1] : p[2];
                tmp0[k] = base + (p[3] * (1.0 - ORA_EXP(p[4] * d->LAI0[(size_t)m * N0 + k])));
            }
            for (int k = 0; k < N1; ++k)
                o->petLAIcorFactor[(size_t)m * N1 + k] = upscale_harm(d, k, tmp0);
        }
        for (int k = 0; k < N1; ++k) {
            o->fAsp[k] = 0.0;
            o->HarSamCoeff[k] = 0.0;
        }
    } else if (d->proc_pet == 3) {
        /* ---- Penman-Monteith resistances per LAI month: aerodynamical_resistance
         * (src/MPR/mo_multi_param_reg.f90:1165-1262, parameters 1-6) and
         * bulksurface_resistance (src/MPR/mo_mpr_pet.f90:407-475, parameter 7),
         * each the arithmetic block mean of its L0 field ---- */
        const double *p = g->pet;
        const double zm_meas = 10.0, karman = 0.41; /* WindMeasHeight, karman (mo_mpr_constants.f90:65-67) */
        const double nodata = -9999.0;
        double *hc0 = (double *)malloc((size_t)N0 * sizeof(double));
        double *maxlai = (double *)malloc((size_t)N0 * sizeof(double));
        if (!hc0 || !maxlai) {
            free(hc0);
            free(maxlai);
            rc = -2;
            goto done;
        }
        for (int k = 0; k < N0; ++k) {
            const int lc = d->LCover0[k];
            hc0[k] = lc == 1 ? p[0] : (lc == 2 ? p[1] : nodata); /* forest, impervious */
            double mx = d->LAI0[k];                                  /* MAXVAL(LAI0, dim=2) */
            for (int m = 1; m < nLAI; ++m)
                if (d->LAI0[(size_t)m * N0 + k] > mx) mx = d->LAI0[(size_t)m * N0 + k];
            maxlai[k] = mx;
        }
        for (int m = 0; m < nLAI; ++m) {
            for (int k = 0; k < N0; ++k) {
                const double lai = d->LAI0[(size_t)m * N0 + k];
                if (d->LCover0[k] == 3) hc0[k] = p[2] * lai / maxlai[k]; /* pervious: the month's LAI */
                double zm = zm_meas;
                if (fabs(zm - nodata) > DBL_EPSILON && zm < hc0[k]) zm = hc0[k] + zm;
                const double displace = p[3] * hc0[k];
                const double zm_zero = p[4] * hc0[k];
                const double zh_zero = p[5] * zm_zero;
                tmp0[k] = ORA_LOG((zm - displace) / zm_zero) * ORA_LOG((zm - displace) / zh_zero) /
                          (karman * karman);
            }
            for (int k = 0; k < N1; ++k)
                o->aeroResist[(size_t)m * N1 + k] = upscale_arith(d, k, tmp0);
            for (int k = 0; k < N0; ++k) {
                const double lai = d->LAI0[(size_t)m * N0 + k];
                double r = p[6] / (lai / (0.3 * lai + 1.2)); /* LAI_factor/offset_surfResi */
                tmp0[k] = r > 250.0 ? 250.0 : r;             /* max_surfResist */
            }
            for (int k = 0; k < N1; ++k)
                o->surfResist[(size_t)m * N1 + k] = upscale_arith(d, k, tmp0);
        }
        free(hc0);
        free(maxlai);
        for (int k = 0; k < N1; ++k) {
            o->fAsp[k] = 0.0;
            o->HarSamCoeff[k] = 0.0;
        }
        if (o->petLAIcorFactor)
            for (size_t i = 0; i < (size_t)nLAI * N1; ++i)
                o->petLAIcorFactor[i] = 0.0;
    } else if (d->proc_pet == 2) {
        /* ---- Priestley-Taylor alpha, src/MPR/mo_mpr_pet.f90:311-369: arithmetic
         * block mean of alpha0 = p1 + p2 * LAI0 per LAI month ---- */
        const double *p = g->pet;
        for (int m = 0; m < nLAI; ++m) {
            for (int k = 0; k < N0; ++k)
                tmp0[k] = p[0] + p[1] * d->LAI0[(size_t)m * N0 + k];
            for (int k = 0; k < N1; ++k)
                o->PrieTayAlpha[(size_t)m * N1 + k] = upscale_arith(d, k, tmp0);
        }
        for (int k = 0; k < N1; ++k) {
            o->fAsp[k] = 0.0; /* not regionalised for this PET process */
            o->HarSamCoeff[k] = 0.0;
        }
        if (o->petLAIcorFactor)
            for (size_t i = 0; i < (size_t)nLAI * N1; ++i)
                o->petLAIcorFactor[i] = 0.0;
    } else {
        /* ---- PET correction by aspect, src/MPR/mo_mpr_pet.f90:214-272 ---- */
        const double *p = g->pet;
        double tmax = p[0] + p[1];
        for (int k = 0; k < N0; ++k) {
            double asp = d->Asp0[k];
            double nth = (asp < p[2]) ? p[0] + (tmax - p[0]) / p[2] * asp
                                      : p[0] + (tmax - p[0]) / (360.0 - p[2]) * (360.0 - asp);
            double sth = (asp < p[2]) ? p[0] + (tmax - p[0]) / (360.0 - p[2]) * (360.0 - asp)
                                      : p[0] + (tmax - p[0]) / p[2] * asp;
            tmp0[k] = (d->y0[k] > 0.0) ? nth : sth;
        }
        for (int k = 0; k < N1; ++k) {
            o->fAsp[k] = upscale_arith(d, k, tmp0);
            o->HarSamCoeff[k] = (d->proc_pet == 1) ? p[3] : 0.0;
        }
        if (o->petLAIcorFactor)
            for (size_t i = 0; i < (size_t)nLAI * N1; ++i)
                o->petLAIcorFactor[i] = 0.0;
    }
    /* ---- mpr_runoff, src/MPR/mo_mpr_runoff.f90:74-194 ---- */
    {
        const double *p = g->interflow;
        for (int k = 0; k < N0; ++k)
            tmp0[k] = p[0] * SMs_FC0[k];
        for (int k = 0; k < N1; ++k)
            o->unsatThresh[k] = upscale_arith(d, k, tmp0);
        for (int k = 0; k < N0; ++k) {
            tmp0[k] = p[1] * (2.0 - d->slope_emp0[k]);
            if (d->LCover0[k] == 1)
                tmp0[k] = tmp0[k] * p[2];
        }
        for (int k = 0; k < N1; ++k) {
            o->kFastFlow[k] = upscale_arith(d, k, tmp0);
            if (o->kFastFlow[k] < 1.0)
                o->kFastFlow[k] = 1.0;
        }
        for (int k = 0; k < N0; ++k)
            tmp0[k] = p[1] * (2.0 - d->slope_emp0[k]) + p[3] * (1.0 + KsVar_H0[k]);
        for (int k = 0; k < N1; ++k) {
            o->kSlowFlow[k] = upscale_arith(d, k, tmp0);
            if (o->kSlowFlow[k] < 2.0)
                o->kSlowFlow[k] = 2.0;
        }
        for (int k = 0; k < N0; ++k)
            tmp0[k] = p[4] * (1.0 / KsVar_H0[k]) * (1.0 / (1.0 + SMs_FC0[k]));
        for (int k = 0; k < N1; ++k) {
            o->alpha[k] = upscale_arith(d, k, tmp0);
            if (o->kFastFlow[k] > o->kSlowFlow[k])
                o->kFastFlow[k] = o->kSlowFlow[k];
        }
    }
    /* ---- karstic_layer, src/MPR/mo_multi_param_reg.f90:944-1036 ---- */
    {
        const double *p = g->perc;
        for (int k = 0; k < N0; ++k)
            tmp0[k] = p[0] * (1.0 + SMs_FC0[k]) / (1.0 + KsVar_V0[k]);
        for (int k = 0; k < N1; ++k) {
            o->kPerco[k] = upscale_arith(d, k, tmp0);
            if (o->kPerco[k] < 2.0)
                o->kPerco[k] = 2.0;
            double fkar = 0.0;
            for (int i = 0; i < d->nGeo; ++i)
                if (d->geoUnitKar[i] != 0)
                    fkar = fraction_cover(d, k, d->geoUnit0, d->geoUnitList[i]); /* the last karstic unit wins */
            o->karstLoss[k] = 1.0 - (fkar * p[1]);
        }
    }
    /* ---- sealed threshold (iper_thres_runoff, :883-894) ---- */
    for (int k = 0; k < N1; ++k)
        o->sealedThresh[k] = g->runoff[0];
    /* ---- baseflow_param (:689-727) and kBaseFlow >= kSlowFlow (:618) ---- */
    for (int k = 0; k < N0; ++k) {
        int best = 0, bd = abs(d->geoUnitList[0] - d->geoUnit0[k]);
        for (int i = 1; i < d->nGeo; ++i) {
            int dd = abs(d->geoUnitList[i] - d->geoUnit0[k]);
            if (dd < bd) {
                bd = dd;
                best = i;
            }
        }
        tmp0[k] = g->geo[best];
    }
    for (int k = 0; k < N1; ++k) {
        o->kBaseFlow[k] = upscale_arith(d, k, tmp0);
        if (o->kBaseFlow[k] < o->kSlowFlow[k])
            o->kBaseFlow[k] = o->kSlowFlow[k];
    }
    /* ---- canopy_intercept_param (:1076-1159) ---- */
    for (int m = 0; m < nLAI; ++m) {
        for (int k = 0; k < N0; ++k)
            tmp0[k] = d->LAI0[(size_t)m * N0 + k] * g->interc[0];
        for (int k = 0; k < N1; ++k)
            o->maxInter[(size_t)m * N1 + k] = upscale_arith(d, k, tmp0);
    }
done:
    free(KsVar_H0); free(KsVar_V0); free(SMs_FC0); free(tmp0); free(t1); free(t2); free(t3); free(t4); free(t5);
    free(Ks); free(Db); free(thS_t); free(thFC_t); free(thPW_t); free(thS); free(thFC); free(thPW);
    free(fForest); free(fPerm);
    return rc;
}

/* generate_soil_database Wd weights, src/MPR/mo_soil_database.f90:387-518
 * (iFlag_soilDB = 0).  horizonDepth[nH-1] is overwritten per soil type with
 * its RZdepth, as the reference does; the value left is the last type's. */
int ora_soil_weights(int nSoil, int maxHor, const int32_t *nHor, const double *UD, const double *LD,
                     const double *RZdepth, int nH, double *horizonDepth, double *Wd)
{
    const double small = 0.000001, acc = 0.5;
    int maxn = 0;
    for (int s = 0; s < nSoil; ++s)
        if (nHor[s] > maxn)
            maxn = nHor[s];
    for (size_t i = 0; i < (size_t)nSoil * nH * maxHor; ++i)
        Wd[i] = 0.0;
    for (int ii = 0; ii < nSoil; ++ii) {
        double *W = Wd + (size_t)ii * nH * maxHor;
        for (int jj = 0; jj < nH; ++jj)
            for (int kk = nHor[ii]; kk < maxn; ++kk)
                W[(size_t)jj * maxHor + kk] = NODATA_DP;
        horizonDepth[nH - 1] = RZdepth[ii];
        for (int jj = 0; jj < nH; ++jj) {
            double *w = W + (size_t)jj * maxHor;
            double dpth_f = (jj != 0) ? horizonDepth[jj - 1] : 0.0;
            double dpth_t = horizonDepth[jj] - acc;
            int lf = -1, lt = -1;
            for (int kk = 0; kk < nHor[ii]; ++kk) {
                double ud = UD[(size_t)ii * maxHor + kk], ld = LD[(size_t)ii * maxHor + kk];
                if (dpth_f >= ud && dpth_f <= (ld - acc))
                    lf = kk;
                if (dpth_t >= ud && dpth_t <= (ld - acc))
                    lt = kk;
            }
            if (lf < 0 || lt < 0 || lf > lt)
                return -(ii + 1);
            if (lf == lt) {
                w[lf] = 1.0;
            } else {
                w[lf] = LD[(size_t)ii * maxHor + lf] - dpth_f;
                w[lt] = (dpth_t + acc) - UD[(size_t)ii * maxHor + lt];
                for (int kk = lf + 1; kk < lt; ++kk)
                    w[kk] = LD[(size_t)ii * maxHor + kk] - UD[(size_t)ii * maxHor + kk];
                double den = (jj != 0) ? (horizonDepth[jj] - horizonDepth[jj - 1]) : horizonDepth[jj];
                for (int kk = 0; kk < nHor[ii]; ++kk)
                    w[kk] = w[kk] / den;
                double s = 0.0;
                for (int kk = 0; kk < maxHor; ++kk)
                    if (w[kk] > 0.0)
                        s = s + w[kk];
                if (s <= 1.0 - small || s >= 1.0 + small)
                    return -(1000 + ii);
            }
        }
    }
    return 0;
}

/* empirical slope distribution, L0_variable_init (src/MPR/mo_mpr_startup.f90:
 * 237-337): rank / (n + 1) in ascending slope order, ties (FORCES eq: relative
 * difference within epsilon) share the value of the later element. */
static const double *g_sort_keys;
static int cmp_idx(const void *a, const void *b)
{
    int ia = *(const int *)a, ib = *(const int *)b;
    double x = g_sort_keys[ia], y = g_sort_keys[ib];
    if (x < y) return -1;
    if (x > y) return 1;
    return (ia > ib) - (ia < ib);
}

int ora_slope_emp(int n, const double *slope, double *slope_emp)
{
    int *idx = (int *)malloc(sizeof(int) * (size_t)n);
    if (!idx)
        return -2;
    for (int i = 0; i < n; ++i)
        idx[i] = i;
    g_sort_keys = slope;
    qsort(idx, (size_t)n, sizeof(int), cmp_idx);
    slope_emp[idx[n - 1]] = (double)n / (double)(n + 1);
    for (int i = n - 2; i >= 0; --i) {
        int is = idx[i], ip = idx[i + 1];
        double a = slope[is], b = slope[ip];
        int eq = !((DBL_EPSILON * fabs(b) - fabs(a - b)) < 0.0); /* FORCES equal_dp */
        slope_emp[is] = eq ? slope_emp[ip] : (double)(i + 1) / (double)(n + 1);
    }
    free(idx);
    return 0;
}
