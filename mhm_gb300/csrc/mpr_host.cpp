// mpr_host.cpp -- parameter-independent MPR start-up on the host (runs once
// per basin; everything that depends on the global parameters runs on the
// device in mpr.cu).
#include "mpr_host.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <numeric>

namespace mhm {

bool soil_weights(int32_t n_soil, int32_t max_hor, const int32_t *n_hor, const double *ud, const double *ld,
                  const double *rz, int32_t H, double *hd, double *Wd, std::string &err)
{
    const double small = 0.000001, acc = 0.5; // src/MPR/mo_soil_database.f90:408-409
    int32_t maxn = 0;
    double dmin = HUGE_VAL;
    for (int32_t s = 0; s < n_soil; ++s) {
        if (n_hor[s] < 1 || n_hor[s] > max_hor) {
            err = "soil type " + std::to_string(s + 1) + ": horizon count out of range";
            return false;
        }
        maxn = std::max(maxn, n_hor[s]);
        if (rz[s] > 0.0 && rz[s] < dmin) dmin = rz[s];
    }
    // :414-422 -- the modelled horizons must end above the shallowest soil
    if (H >= 2 && hd[H - 2] >= dmin) {
        err = "horizon depths reach below the shallowest soil type (generate_soil_database)";
        return false;
    }
    std::fill(Wd, Wd + (size_t)n_soil * H * max_hor, 0.0);
    for (int32_t s = 0; s < n_soil; ++s) {
        double *W = Wd + (size_t)s * H * max_hor;
        for (int32_t h = 0; h < H; ++h)
            for (int32_t k = n_hor[s]; k < maxn; ++k) W[(size_t)h * max_hor + k] = -9999.0;
        hd[H - 1] = rz[s];
        const double *U = ud + (size_t)s * max_hor, *D = ld + (size_t)s * max_hor;
        for (int32_t h = 0; h < H; ++h) {
            double *w = W + (size_t)h * max_hor;
            const double dpth_f = (h != 0) ? hd[h - 1] : 0.0;
            const double dpth_t = hd[h] - acc;
            int32_t lf = -1, lt = -1;
            for (int32_t k = 0; k < n_hor[s]; ++k) {
                if (dpth_f >= U[k] && dpth_f <= (D[k] - acc)) lf = k;
                if (dpth_t >= U[k] && dpth_t <= (D[k] - acc)) lt = k;
            }
            if (lf < 0 || lt < 0 || lf > lt) {
                err = "horizon depths do not lie in the database for soil type " + std::to_string(s + 1);
                return false;
            }
            if (lf == lt) {
                w[lf] = 1.0;
                continue;
            }
            w[lf] = D[lf] - dpth_f;
            w[lt] = (dpth_t + acc) - U[lt];
            for (int32_t k = lf + 1; k < lt; ++k) w[k] = D[k] - U[k];
            const double den = (h != 0) ? (hd[h] - hd[h - 1]) : hd[h];
            for (int32_t k = 0; k < n_hor[s]; ++k) w[k] = w[k] / den;
            double sum = 0.0;
            for (int32_t k = 0; k < max_hor; ++k)
                if (w[k] > 0.0) sum = sum + w[k];
            if (sum <= 1.0 - small || sum >= 1.0 + small) {
                err = "soil horizon weights do not sum to 1 for soil type " + std::to_string(s + 1);
                return false;
            }
        }
    }
    return true;
}

void slope_empirical(int32_t n, const double *slope, double *se)
{
    if (n <= 0) return;
    std::vector<int32_t> idx(n);
    std::iota(idx.begin(), idx.end(), 0);
    std::sort(idx.begin(), idx.end(), [slope](int32_t a, int32_t b) {
        return slope[a] < slope[b] || (slope[a] == slope[b] && a < b);
    });
    se[idx[n - 1]] = (double)n / (double)(n + 1);
    for (int32_t i = n - 2; i >= 0; --i) {
        const int32_t is = idx[i], ip = idx[i + 1];
        const double a = slope[is], b = slope[ip];
        // equality within relative machine epsilon, as mo_utils' eq
        const bool eq = !((DBL_EPSILON * std::fabs(b) - std::fabs(a - b)) < 0.0);
        se[is] = eq ? se[ip] : (double)(i + 1) / (double)(n + 1);
    }
}

bool mpr_prepare(const mhm_l0_desc &l0, int32_t n1, int32_t H, MprSetup &o, std::string &err)
{
    const int32_t n0 = l0.n_cells0, nr = l0.nrows0, nc = l0.ncols0;
    if (n0 <= 0 || nr <= 0 || nc <= 0 || !l0.mask0 || !l0.soil_id0 || !l0.lcover0 || !l0.geo_unit0 ||
        !l0.slope0 || !l0.aspect0 || !l0.y0 || !l0.l1_up || !l0.l1_down || !l0.l1_left || !l0.l1_right ||
        !l0.l1_nsub || !l0.horizon_depth || !l0.soil_n_hor || !l0.soil_n_till || !l0.soil_ud || !l0.soil_ld ||
        !l0.soil_sand || !l0.soil_clay || !l0.soil_dbm || !l0.soil_rz_depth || !l0.geo_unit_list ||
        !l0.geo_unit_kar) {
        err = "L0 description incomplete";
        return false;
    }
    if (H < 2) {
        err = "MPR needs at least 2 soil horizons (the last one ends at the soil's RZdepth)";
        return false;
    }
    if (l0.n_soil_types < 1 || (int64_t)l0.n_soil_types * 3 > (int64_t)kMprKeyMask + 1 || l0.max_soil_hor < 1 ||
        l0.n_geo_units < 1 || l0.n_geo_units > 256 || l0.n_lai_classes < 0 || l0.n_lai_classes > 256) {
        err = "soil, geology or LAI class counts out of range";
        return false;
    }
    if (l0.n_lai_classes > 0 ? (!l0.lai_class0 || !l0.lai_lut) : !l0.lai0) {
        err = "LAI input missing";
        return false;
    }
    if (l0.n_lai_steps < 0 || l0.n_lai_steps > 32767 || (l0.n_lai_classes > 0 && l0.n_lai_steps != 0 &&
                                                        l0.n_lai_steps != 12)) {
        err = "LAI entries out of range (a look-up table has 12 monthly entries)";
        return false;
    }
    o.n1 = n1;
    o.n0 = n0;
    o.H = H;
    o.n_soil = l0.n_soil_types;
    o.max_hor = l0.max_soil_hor;
    o.n_keys = 3 * o.n_soil;
    o.n_lai_classes = l0.n_lai_classes;
    o.n_lai_steps = (l0.n_lai_classes > 0 || l0.n_lai_steps == 0) ? 12 : l0.n_lai_steps;
    o.n_geo = l0.n_geo_units;
    const size_t nsh = (size_t)o.n_soil * o.max_hor;
    o.n_hor.assign(l0.soil_n_hor, l0.soil_n_hor + o.n_soil);
    o.n_till.assign(l0.soil_n_till, l0.soil_n_till + o.n_soil);
    o.sand.assign(l0.soil_sand, l0.soil_sand + nsh);
    o.clay.assign(l0.soil_clay, l0.soil_clay + nsh);
    o.dbm.assign(l0.soil_dbm, l0.soil_dbm + nsh);
    o.rz.assign(l0.soil_rz_depth, l0.soil_rz_depth + o.n_soil);
    for (int32_t s = 0; s < o.n_soil; ++s)
        if (o.n_till[s] < 1 || o.n_till[s] > o.n_hor[s]) {
            err = "soil type " + std::to_string(s + 1) + ": tillage horizon count out of range";
            return false;
        }
    o.horizon_depth.assign(l0.horizon_depth, l0.horizon_depth + H);
    o.Wd.assign((size_t)o.n_soil * H * o.max_hor, 0.0);
    if (!soil_weights(o.n_soil, o.max_hor, l0.soil_n_hor, l0.soil_ud, l0.soil_ld, l0.soil_rz_depth, H,
                      o.horizon_depth.data(), o.Wd.data(), err))
        return false;
    o.slope_emp.assign(n0, 0.0);
    slope_empirical(n0, l0.slope0, o.slope_emp.data());
    if (o.n_lai_classes > 0) o.lai_lut.assign(l0.lai_lut, l0.lai_lut + (size_t)o.n_lai_classes * 12);

    // L0 cell id of every grid position (column-major packing over mask0)
    std::vector<int32_t> id2d((size_t)nr * nc, -1);
    int32_t k0 = 0;
    for (size_t p = 0; p < id2d.size(); ++p)
        if (l0.mask0[p]) id2d[p] = k0++;
    if (k0 != n0) {
        err = "mask0 holds " + std::to_string(k0) + " cells, n_cells0 = " + std::to_string(n0);
        return false;
    }
    o.present.assign(o.n_soil, 0);
    std::vector<uint32_t> code0(n0);
    for (int32_t k = 0; k < n0; ++k) {
        const int32_t s = l0.soil_id0[k], lc = l0.lcover0[k];
        if (s < 1 || s > o.n_soil || lc < 1 || lc > 3) {
            err = "L0 cell " + std::to_string(k + 1) + ": soil or land-cover id out of range";
            return false;
        }
        o.present[s - 1] = 1;
        uint32_t c = (uint32_t)((s - 1) * 3 + (lc - 1));
        if (l0.y0[k] > 0.0) c |= kMprNorth;
        if (lc == 1) c |= kMprForest;
        if (o.n_lai_classes > 0) {
            const int32_t lai = l0.lai_class0[k];
            if (lai < 1 || lai > o.n_lai_classes) {
                err = "L0 cell " + std::to_string(k + 1) + ": LAI class out of range";
                return false;
            }
            c |= (uint32_t)(lai - 1) << 16;
        }
        // baseflow_param (src/MPR/mo_multi_param_reg.f90:689-727): the first
        // unit of GeoUnitList with the smallest |unit - geoUnit0|
        int32_t best = 0, bd = std::abs(l0.geo_unit_list[0] - l0.geo_unit0[k]);
        for (int32_t i = 1; i < o.n_geo; ++i) {
            const int32_t d = std::abs(l0.geo_unit_list[i] - l0.geo_unit0[k]);
            if (d < bd) {
                bd = d;
                best = i;
            }
        }
        c |= (uint32_t)best << 24;
        code0[k] = c;
    }
    o.dpth_t_last = o.rz[l0.soil_id0[n0 - 1] - 1];

    // sub-cell slots of every L1 cell: its L0 cells in the column-major
    // order of the reference's masked block sums
    o.nsub.assign(n1, 0);
    o.f_forest.assign(n1, 0.0);
    o.f_sealed.assign(n1, 0.0);
    o.f_perm.assign(n1, 0.0);
    o.f_kar.assign(n1, 0.0);
    int32_t max_sub = 0;
    for (int32_t k = 0; k < n1; ++k) {
        const int32_t iu = l0.l1_up[k], id = l0.l1_down[k], jl = l0.l1_left[k], jr = l0.l1_right[k];
        if (iu < 1 || id > nr || jl < 1 || jr > nc || iu > id || jl > jr) {
            err = "L1 cell " + std::to_string(k + 1) + ": L0 bounds out of range";
            return false;
        }
        int32_t n = 0;
        for (int32_t j = jl; j <= jr; ++j)
            for (int32_t i = iu; i <= id; ++i)
                if (id2d[(size_t)(j - 1) * nr + (i - 1)] >= 0) ++n;
        if (n != l0.l1_nsub[k] || n == 0) {
            err = "L1 cell " + std::to_string(k + 1) + ": n_subcells does not match mask0";
            return false;
        }
        o.nsub[k] = n;
        max_sub = std::max(max_sub, n);
    }
    o.max_sub = max_sub;
    const size_t slots = (size_t)max_sub * n1;
    o.sub_code.assign(slots, 0u);
    o.sub_se.assign(slots, 0.0);
    o.sub_asp.assign(slots, 0.0);
    if (o.n_lai_classes == 0) o.sub_lai.assign((size_t)o.n_lai_steps * slots, 0.0);
    for (int32_t k = 0; k < n1; ++k) {
        const int32_t iu = l0.l1_up[k], id = l0.l1_down[k], jl = l0.l1_left[k], jr = l0.l1_right[k];
        int32_t slot = 0, c_forest = 0, c_sealed = 0;
        for (int32_t j = jl; j <= jr; ++j)
            for (int32_t i = iu; i <= id; ++i) {
                const int32_t c = id2d[(size_t)(j - 1) * nr + (i - 1)];
                if (c < 0) continue;
                const size_t p = (size_t)slot * n1 + k;
                o.sub_code[p] = code0[c];
                o.sub_se[p] = o.slope_emp[c];
                o.sub_asp[p] = l0.aspect0[c];
                if (o.n_lai_classes == 0)
                    for (int m = 0; m < o.n_lai_steps; ++m)
                        o.sub_lai[(size_t)m * slots + p] = l0.lai0[(size_t)m * n0 + c];
                c_forest += (l0.lcover0[c] == 1);
                c_sealed += (l0.lcover0[c] == 2);
                ++slot;
            }
        // L0_fractionalCover_in_Lx and the sealed-fraction update
        // (src/MPR/mo_multi_param_reg.f90:273-297)
        const double n = (double)o.nsub[k];
        o.f_forest[k] = (double)c_forest / n;
        o.f_sealed[k] = l0.frac_sealed_city * ((double)c_sealed / n);
        o.f_perm[k] = 1.0 - o.f_sealed[k] - o.f_forest[k];
        // karstic_layer (:1024-1029): the last karstic unit of the list wins
        for (int32_t g = 0; g < o.n_geo; ++g) {
            if (l0.geo_unit_kar[g] == 0) continue;
            int32_t cnt = 0;
            for (int32_t j = jl; j <= jr; ++j)
                for (int32_t i = iu; i <= id; ++i) {
                    const int32_t c = id2d[(size_t)(j - 1) * nr + (i - 1)];
                    if (c >= 0 && l0.geo_unit0[c] == l0.geo_unit_list[g]) ++cnt;
                }
            o.f_kar[k] = (double)cnt / n;
        }
    }
    return true;
}

} // namespace mhm
