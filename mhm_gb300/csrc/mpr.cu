// mpr.cu -- the multiscale parameter regionalisation (mpr(),
// src/MPR/mo_multi_param_reg.f90:67-654) on the device, per member.
//
// Everything the reference evaluates per L0 cell from the soil database is a
// function of the cell's (soil type, land cover) pair alone: the transfer
// functions, the depth-weighted horizon properties, the root fractions and
// the Ks variabilities.  So the first kernel evaluates them once per pair and
// member into a small table (tens of rows instead of millions of L0 cells);
// the second kernel gives every L1 cell one thread that walks its L0
// sub-cells in the reference's column-major block order and forms the
// arithmetic and harmonic means from table rows and the few per-cell inputs
// (slope rank, aspect, LAI, geology), writing the member's effective
// parameters in place.  The per-cell values are the same IEEE operations on
// the same operands as the reference's per-cell loop, and every block sum
// keeps the reference's order, so results are bit-identical.
#include <cfloat>
#include <cmath>

#include "hmath.h"
#include "bounds.cuh"
#include "mhm_kernels.cuh"
#include "mpr_host.h"

namespace mhm {

namespace {

// src/MPR/mo_mpr_constants.f90:34-62
constexpr double kBulkDensOrgMatter = 0.224, kFieldCapC1 = -0.60, kFieldCapC2 = 2.0, kVGSandThresh = 66.5;
__device__ constexpr double kVGN[18] = {1.392, 0.418, -0.024, 1.212, -0.704, -0.648, 0.023, 0.044, 3.168,
                             -2.562, 7.0E-9, 4.004, 3.750, -0.016, -4.197, 0.013, 0.076, 0.276};
constexpr double kKsC = 10.0, kPwpC = 1.0, kPwpMatPot = 15000.0;

// hydro_cond, src/MPR/mo_mpr_soilmoist.f90:736-772
__device__ double hydro_cond(const double *p, double sand, double clay)
{
    const double x = p[0] + p[1] * sand - p[2] * clay;
    double ks = p[3] * hm_exp(x * hm_log(kKsC));
    return (ks < 1.10) ? 1.10 : ks;
}

// Genuchten, :626-698
__device__ void genuchten(const double *p, double sand, double clay, double db, double &ths, double &n,
                          double &alpha)
{
    double x;
    if (sand < kVGSandThresh) {
        ths = p[0] + p[1] * clay + p[2] * db;
        n = kVGN[0] - kVGN[1] * hm_pow(sand, kVGN[2]) + kVGN[3] * hm_pow(clay, kVGN[4]);
        x = kVGN[5] + kVGN[6] * sand + kVGN[7] * clay - kVGN[8] * db;
    } else {
        ths = p[3] + p[4] * clay + p[5] * db;
        n = kVGN[9] + kVGN[10] * hm_pow(sand, kVGN[11]) + kVGN[12] * hm_pow(clay, kVGN[13]);
        x = kVGN[14] + kVGN[15] * sand + kVGN[16] * clay - kVGN[17] * db;
    }
    alpha = hm_exp(x);
    if (ths < 0.01) ths = 0.01;
    if (ths > 1.0) ths = 1.0;
    if (n < 1.01000) n = 1.01000;
    if (alpha < 0.00001) alpha = 0.00001;
}

// field_cap, :560-584
__device__ double field_cap(double ks, double ths, double n)
{
    const double x = (kFieldCapC1) * (kFieldCapC2 + hm_log10(ks));
    return ths * hm_exp(x * hm_log(n));
}

// PWP, :489-520
__device__ double pwp(double n, double alpha, double ths)
{
    const double m = kPwpC - (kPwpC / n);
    double x = kPwpC + hm_exp(n * hm_log(alpha * kPwpMatPot));
    x = hm_exp(m * hm_log(x));
    if (x < 1.0) x = 1.0;
    return ths / x;
}

// One table row: soil type s, land cover l (0 forest, 1 sealed, 2 pervious).
// mpr_sm (src/MPR/mo_mpr_soilmoist.f90:264-392) for the soil's horizons and
// the pair's L0 quantities, then mpr_SMhorizons (src/MPR/mo_mpr_smhorizons.f90:
// 340-582) for each model horizon; harmonic-mean operands are stored as the
// reciprocals the upscaling sums.
__device__ void soil_row(const MprArgs &a, const double *g, int s, int l, double *row)
{
    const int H = a.H, mh = a.max_hor, nh = a.n_hor[s], nt = a.n_till[s];
    const double *ps = g + a.off.soil;
    const double om_forest = (a.proc_sm <= 2) ? ps[2] + ps[0] : ps[0];
    const double pom = (l == 0) ? om_forest : (l == 1) ? ps[1] : ps[2];
    double ths[kMprMaxSoilHor], thfc[kMprMaxSoilHor], thpw[kMprMaxSoilHor], ks[kMprMaxSoilHor],
        db[kMprMaxSoilHor];
    for (int j = 0; j < nh; ++j) {
        const double sand = a.sand[s * mh + j], clay = a.clay[s * mh + j], dbm = a.dbm[s * mh + j];
        double k = hydro_cond(ps + 9, sand, clay), n, alpha;
        if (j < nt) {
            const double pm = 100.0 - pom;
            db[j] = 100.0 / ((pom / kBulkDensOrgMatter) + (pm / dbm));
            k = k * (dbm / db[j]);
            genuchten(ps + 3, sand, clay, db[j], ths[j], n, alpha);
        } else {
            db[j] = dbm;
            genuchten(ps + 3, sand, clay, dbm, ths[j], n, alpha);
        }
        ks[j] = k;
        thfc[j] = field_cap(k, ths[j], n);
        thpw[j] = pwp(n, alpha, ths[j]);
    }
    // Ks variabilities over the column (:330-352)
    double kh = 0.0, kv = 0.0, fc = 0.0, tot = 0.0;
    for (int j = 0; j < nh; ++j) {
        kh = kh + ths[j] * ks[j];
        kv = kv + ths[j] / ks[j];
        fc = fc + thfc[j];
        tot = tot + ths[j];
    }
    const double sms_fc = (tot - fc) / tot;
    const double ksvar_h = kh / tot / ps[12];
    const double ksvar_v = tot / kv / ps[12];

    // horizons (mpr_SMhorizons); its 4 or 8 parameters follow the first 13
    const double *p2 = ps + 13;
    const double rc_forest = p2[0], rc_imp = p2[1];
    double rc_perv = 0.0, rc_sand = 0.0, rc_clay = 0.0, fcmin = 0.0, fcmax = 0.0;
    if (a.proc_sm <= 2) {
        rc_perv = p2[0] - p2[2];
    } else {
        rc_perv = p2[2];
        rc_sand = p2[5] - p2[4];
        rc_clay = p2[5];
        fcmin = p2[6];
        fcmax = p2[6] + p2[7];
    }
    for (int h = 0; h < H; ++h) {
        const double *wd = a.Wd + ((size_t)s * H + h) * mh;
        double a1 = 0.0, b1 = 0.0;
        for (int j = 0; j < nt; ++j)
            if (wd[j] > 0.0) a1 = a1 + db[j] * wd[j];
        for (int j = nt; j < nh; ++j)
            if (wd[j] >= 0.0) b1 = b1 + db[j] * wd[j];
        const double bd = a1 + b1;
        double sums[3];
        const double *th[3] = {ths, thfc, thpw};
        for (int q = 0; q < 3; ++q) {
            double x = 0.0, y = 0.0;
            for (int j = 0; j < nt; ++j)
                if (wd[j] > 0.0) x = x + th[q][j] * wd[j];
            for (int j = nt; j < nh; ++j)
                if (wd[j] > 0.0) y = y + th[q][j] * wd[j];
            sums[q] = x + y;
        }
        double dpth_f = 0.0, dpth_t = a.hd[h];
        if (h > 0 && h < H - 1) dpth_f = a.hd[h - 1];
        double dpth_t_roots = dpth_t;
        if (h == H - 1) {
            dpth_f = a.hd[H - 2];
            dpth_t = a.rz[s];               // this cell's own soil
            dpth_t_roots = a.dpth_t_last;   // what the root loop sees afterwards
        }
        const double sms = sums[0] * (dpth_t - dpth_f);
        const double fcv = sums[1] * (dpth_t - dpth_f);
        const double pwv = sums[2] * (dpth_t - dpth_f);
        double c;
        if (l == 0) {
            c = rc_forest;
        } else if (l == 1) {
            c = rc_imp;
        } else if (a.proc_sm <= 2) {
            c = rc_perv;
        } else {
            double fcn = (((fcv / (dpth_t_roots - dpth_f)) - fcmin) / (fcmax - fcmin));
            if (fcn < 0.0)
                fcn = 0.0;
            else if (fcn > 1.0)
                fcn = 1.0;
            c = (fcn * rc_clay) + ((1.0 - fcn) * rc_sand);
        }
        const double fr = (1.0 - hm_pow(c, dpth_t_roots * 0.1)) - (1.0 - hm_pow(c, dpth_f * 0.1));
        row[MT_INV_SMS * H + h] = 1.0 / sms;
        row[MT_INV_BETA * H + h] = 1.0 / (bd * p2[3]);
        row[MT_INV_PW * H + h] = 1.0 / pwv;
        row[MT_INV_FC * H + h] = 1.0 / fcv;
        row[MT_INV_FROOTS * H + h] = 1.0 / fr;
    }
    const double *pi = g + a.off.interflow, *pp = g + a.off.perc;
    row[5 * H + 0] = pi[0] * sms_fc;                                      // mpr_runoff HL1 operand
    row[5 * H + 1] = pi[3] * (1.0 + ksvar_h);                             // K1 soil term
    row[5 * H + 2] = pi[4] * (1.0 / ksvar_h) * (1.0 / (1.0 + sms_fc));    // alpha operand
    row[5 * H + 3] = pp[0] * (1.0 + sms_fc) / (1.0 + ksvar_v);            // karstic_layer Kp operand
}

// grid (ceil(rows / 64), members): soil rows, then (proc_pet = -1 with class
// LAI) the reciprocal LAI correction factors of pet_correctbyLAI
// (src/MPR/mo_mpr_pet.f90:60-140) per (land cover, LAI class, month)
__global__ void __launch_bounds__(64) mpr_table_kernel(MprArgs a)
{
    const int m = blockIdx.y;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const double *g = a.gamma + (size_t)m * a.n_gamma;
    const int ts = mpr_table_stride(a.H);
    if (t < a.n_keys) {
        soil_row(a, g, t / 3, t % 3, a.table + ((size_t)m * a.n_keys + t) * ts);
        return;
    }
    const int u = t - a.n_keys;
    if (a.proc_pet != -1 || a.n_lai_classes == 0 || u >= 3 * a.n_lai_classes * 12) return;
    const int l = u / (a.n_lai_classes * 12), c = (u / 12) % a.n_lai_classes, mo = u % 12;
    const double *p = g + a.off.pet;
    const double base = (l == 0) ? p[0] : (l == 1) ? p[1] : p[2];
    const double f = base + (p[3] * (1.0 - hm_exp(p[4] * a.lai_lut[c * 12 + mo])));
    a.petlai[(size_t)m * 3 * a.n_lai_classes * 12 + u] = 1.0 / f;
}

// grid (ceil(n1 / 128), members): one thread per L1 cell
__global__ void __launch_bounds__(128) mpr_upscale_kernel(MprArgs a)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a.n1) return;
    const int m = blockIdx.y, H = a.H, ts = mpr_table_stride(H);
    const size_t N = a.n1;
    const double *g = a.gamma + (size_t)m * a.n_gamma;
    const double *tab = a.table + (size_t)m * a.n_keys * ts;
    double *out = a.params + (size_t)m * a.member_stride;
    const int ns = a.nsub[k];
    const double dn = (double)ns;
    const uint32_t *code = a.code + k;
    const double *se = a.se + k, *asp = a.asp + k;

    // soil horizons: harmonic means (upscale_harmonic_mean,
    // src/MPR/mo_upscaling_operators.f90:369-432), then the limits and the
    // root normalisation of mpr_SMhorizons (src/MPR/mo_mpr_smhorizons.f90:712-737)
    double froots[kMaxHorizons];
    for (int h = 0; h < H; ++h) {
        double s_sms = 0.0, s_beta = 0.0, s_pw = 0.0, s_fc = 0.0, s_fr = 0.0;
        for (int j = 0; j < ns; ++j) {
            const uint32_t key = __ldg(code + (size_t)j * N) & kMprKeyMask;
            if (!bc_ok(BC_MPR_KEY, key, a.n_keys)) continue;
            const double *row = tab + (size_t)key * ts;
            s_sms = s_sms + __ldg(row + MT_INV_SMS * H + h);
            s_beta = s_beta + __ldg(row + MT_INV_BETA * H + h);
            s_pw = s_pw + __ldg(row + MT_INV_PW * H + h);
            s_fc = s_fc + __ldg(row + MT_INV_FC * H + h);
            s_fr = s_fr + __ldg(row + MT_INV_FROOTS * H + h);
        }
        double sms = dn / s_sms, fc = dn / s_fc, pw = dn / s_pw;
        froots[h] = dn / s_fr;
        if (fc > sms) fc = sms - 0.01 * sms;
        if (pw > fc) pw = fc - 0.01 * fc;
        if (sms < 0.0) sms = 0.0001;
        if (fc < 0.0) fc = 0.0001;
        if (pw < 0.0) pw = 0.0001;
        out[(size_t)(P_HORIZON + 1 * H + h) * N + k] = sms;
        out[(size_t)(P_HORIZON + 2 * H + h) * N + k] = fc;
        out[(size_t)(P_HORIZON + 3 * H + h) * N + k] = pw;
        out[(size_t)(P_HORIZON + 4 * H + h) * N + k] = dn / s_beta;
    }
    double ftot = 0.0;
    for (int h = 0; h < H; ++h)
        if (froots[h] > 0.0) ftot = ftot + froots[h];
    for (int h = 0; h < H; ++h)
        out[(size_t)(P_HORIZON + h) * N + k] = (ftot > 0.0) ? froots[h] / ftot : 0.0;

    // arithmetic means (upscale_arithmetic_mean, :266-329) of mpr_runoff
    // (src/MPR/mo_mpr_runoff.f90:141-191), karstic_layer (Kp), baseflow_param
    // and pet_correctbyASP (src/MPR/mo_mpr_pet.f90:236-272)
    const double *pi = g + a.off.interflow, *pp = g + a.off.pet, *geo = g + a.off.geo;
    const bool asp_on = (a.proc_pet == 0 || a.proc_pet == 1);
    const double tmax = pp[0] + pp[1];
    const double slope_lo = asp_on ? (tmax - pp[0]) / pp[2] : 0.0;
    const double slope_hi = asp_on ? (tmax - pp[0]) / (360.0 - pp[2]) : 0.0;
    double s_hl1 = 0.0, s_k0 = 0.0, s_k1 = 0.0, s_alpha = 0.0, s_kp = 0.0, s_k2 = 0.0, s_asp = 0.0;
    for (int j = 0; j < ns; ++j) {
        const uint32_t c = __ldg(code + (size_t)j * N);
        if (!bc_ok(BC_MPR_KEY, c & kMprKeyMask, a.n_keys) ||
            !bc_ok(BC_MPR_GEO, (long long)(c >> 24), (long long)a.n_gamma - a.off.geo))
            continue;
        const double *row = tab + (size_t)(c & kMprKeyMask) * ts;
        const double sej = __ldg(se + (size_t)j * N);
        s_hl1 = s_hl1 + __ldg(row + 5 * H + 0);
        double t0 = pi[1] * (2.0 - sej);
        if (c & kMprForest) t0 = t0 * pi[2];
        s_k0 = s_k0 + t0;
        s_k1 = s_k1 + (pi[1] * (2.0 - sej) + __ldg(row + 5 * H + 1));
        s_alpha = s_alpha + __ldg(row + 5 * H + 2);
        s_kp = s_kp + __ldg(row + 5 * H + 3);
        s_k2 = s_k2 + geo[c >> 24];
        if (asp_on) {
            const double x = __ldg(asp + (size_t)j * N);
            // northern cells: the low branch below the threshold aspect;
            // southern cells: the mirrored assignment
            const bool low = ((c & kMprNorth) != 0) == (x < pp[2]);
            s_asp = s_asp + (low ? pp[0] + slope_lo * x : pp[0] + slope_hi * (360.0 - x));
        }
    }
    double k0 = s_k0 / dn, k1 = s_k1 / dn, kp = s_kp / dn, k2 = s_k2 / dn;
    if (k0 < 1.0) k0 = 1.0;
    if (k1 < 2.0) k1 = 2.0;
    if (k0 > k1) k0 = k1;
    if (kp < 2.0) kp = 2.0;
    if (k2 < k1) k2 = k1; // src/MPR/mo_multi_param_reg.f90:618
    out[(size_t)P_UTHRESH * N + k] = s_hl1 / dn;
    out[(size_t)P_K0 * N + k] = k0;
    out[(size_t)P_K1 * N + k] = k1;
    out[(size_t)P_ALPHA * N + k] = s_alpha / dn;
    out[(size_t)P_KP * N + k] = kp;
    out[(size_t)P_K2 * N + k] = k2;
    out[(size_t)P_FASP * N + k] = asp_on ? s_asp / dn : 0.0;
    out[(size_t)P_HARSAM * N + k] = (a.proc_pet == 1) ? pp[3] : 0.0;

    // land-cover fractions, snow (snow_acc_melt_param, :800-852), sealed
    // threshold, karst loss (karstic_layer, :1032) and Jarvis threshold
    const double *psn = g + a.off.snow;
    const double ff = a.f_forest[k], fs = a.f_sealed[k], fp = a.f_perm[k];
    const double ddf_f = psn[1], ddf_i = psn[1] + psn[3] + psn[2], ddf_p = psn[1] + psn[3];
    const double mdf_f = psn[1] + psn[5], mdf_i = psn[1] + psn[3] + psn[2] + psn[6], mdf_p = psn[1] + psn[3] + psn[7];
    out[(size_t)P_FSEALED * N + k] = fs;
    out[(size_t)P_TTHRESH * N + k] = psn[0];
    out[(size_t)P_DDINC * N + k] = psn[4];
    out[(size_t)P_DDNOPRE * N + k] = (ddf_f * ff + ddf_i * fs + ddf_p * fp);
    out[(size_t)P_DDMAX * N + k] = (mdf_f * ff + mdf_i * fs + mdf_p * fp);
    out[(size_t)P_STHRESH * N + k] = g[a.off.runoff];
    out[(size_t)P_KARST * N + k] = 1.0 - (a.f_kar[k] * g[a.off.perc + 1]);
    out[(size_t)P_JARVIS * N + k] =
        (a.proc_sm == 2 || a.proc_sm == 3) ? g[a.off.soil + a.off.n_soil_params - 1] : 0.0;

    // canopy_intercept_param (src/MPR/mo_multi_param_reg.f90:1132-1152) and
    // pet_correctbyLAI, per LAI entry (12 monthly slots or a gridded series:
    // the reference loops over size(LAI0, 2), :1142)
    const double gi = g[a.off.interc];
    const size_t slots = (size_t)a.max_sub * N;
    const double *plai = a.petlai + (size_t)m * 3 * a.n_lai_classes * 12;
    const int n_lai = a.n_lai_steps;
    for (int mo = 0; mo < n_lai; ++mo) {
        double s_int = 0.0, s_pet = 0.0, s_pt = 0.0, s_ra = 0.0, s_rs = 0.0;
        for (int j = 0; j < ns; ++j) {
            const uint32_t c = __ldg(code + (size_t)j * N);
            if (!a.lai && !bc_ok(BC_MPR_LAI, (c >> 16) & 0xFFu, a.n_lai_classes)) continue;
            double lai;
            if (a.lai) {
                lai = __ldg(a.lai + mo * slots + (size_t)j * N + k);
            } else {
                lai = __ldg(a.lai_lut + ((c >> 16) & 0xFFu) * 12 + mo);
            }
            s_int = s_int + lai * gi;
            // priestley_taylor_alpha, src/MPR/mo_mpr_pet.f90:311-369: alpha0 = p1 + p2 LAI0
            if (a.proc_pet == 2) s_pt = s_pt + (pp[0] + pp[1] * lai);
            if (a.proc_pet == 3) {
                // aerodynamical_resistance, src/MPR/mo_multi_param_reg.f90:1165-1262: canopy
                // height by land cover (pervious: p3 LAI / max over the months), measurement
                // height 10 m raised above the canopy, log profile with karman = 0.41
                const int l = (int)((c & kMprKeyMask) % 3u); // 0 forest, 1 impervious, 2 pervious
                double hc = (l == 0) ? pp[0] : pp[1];
                if (l == 2) {
                    double mx = -1.0e300;
                    for (int t = 0; t < n_lai; ++t) { // MAXVAL(LAI0, dim=2) over every entry
                        const double x = a.lai ? __ldg(a.lai + t * slots + (size_t)j * N + k)
                                               : __ldg(a.lai_lut + ((c >> 16) & 0xFFu) * 12 + t);
                        mx = (t == 0 || x > mx) ? x : mx;
                    }
                    hc = pp[2] * lai / mx;
                }
                double zm = 10.0;
                if (zm < hc) zm = hc + zm;
                const double disp = pp[3] * hc, z0m = pp[4] * hc, z0h = pp[5] * z0m;
                s_ra = s_ra + hm_log((zm - disp) / z0m) * hm_log((zm - disp) / z0h) / (0.41 * 0.41);
                // bulksurface_resistance, src/MPR/mo_mpr_pet.f90:407-475, capped at 250 s m-1
                const double rs = pp[6] / (lai / (0.3 * lai + 1.2));
                s_rs = s_rs + (rs > 250.0 ? 250.0 : rs);
            }
            if (a.proc_pet == -1) {
                const int l = (int)((c & kMprKeyMask) % 3u);
                double inv;
                if (a.lai) {
                    const double base = (l == 0) ? pp[0] : (l == 1) ? pp[1] : pp[2];
                    inv = 1.0 / (base + (pp[3] * (1.0 - hm_exp(pp[4] * lai))));
                } else {
                    inv = __ldg(plai + ((size_t)l * a.n_lai_classes + ((c >> 16) & 0xFFu)) * 12 + mo);
                }
                s_pet = s_pet + inv;
            }
        }
        const double v_int = s_int / dn;
        const double v_pet = (a.proc_pet == -1) ? dn / s_pet
                             : (a.proc_pet == 2) ? s_pt / dn
                             : (a.proc_pet == 3) ? s_ra / dn : 0.0;
        const double v_pet2 = (a.proc_pet == 3) ? s_rs / dn : 0.0;
        if (a.lai_out) { // a gridded LAI series: [member][lai_groups][n_lai][N]
            const int ng = lai_groups(a.proc_pet);
            double *lo = a.lai_out + (size_t)m * ng * n_lai * N + (size_t)mo * N + k;
            lo[0] = v_int;
            if (ng > 1) lo[(size_t)n_lai * N] = v_pet;
            if (ng > 2) lo[(size_t)2 * n_lai * N] = v_pet2;
        } else {
            out[(size_t)(P_MAXINTER + mo) * N + k] = v_int;
            out[(size_t)(P_PETLAI + mo) * N + k] = v_pet;
            out[(size_t)(P_PET2 + mo) * N + k] = v_pet2;
        }
    }
}

} // namespace

cudaError_t launch_mpr(const MprArgs &a, cudaStream_t s)
{
    if (a.n_members <= 0) return cudaSuccess;
    const int rows = a.n_keys + ((a.proc_pet == -1) ? 3 * a.n_lai_classes * 12 : 0);
    mpr_table_kernel<<<dim3((rows + 63) / 64, a.n_members), 64, 0, s>>>(a);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    mpr_upscale_kernel<<<dim3((a.n1 + 127) / 128, a.n_members), 128, 0, s>>>(a);
    return cudaGetLastError();
}

} // namespace mhm

MHM_BC_ACCESSOR(bc_take_mpr)
