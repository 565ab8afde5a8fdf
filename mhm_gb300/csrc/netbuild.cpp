// netbuild.cpp -- mRM's start-up of the L11 routing network from level-0
// flow data (host code, run once per basin): the L11 grid over the L0 mask,
// the L11 flow directions and outlet cells, the links and their routing
// order, where each link starts and ends on the L0 grid, each link's length,
// slope and floodplain, and the sealed fraction of the floodplains.
//
// Grids use mHM's conventions: a grid (i, j) has i = 1..nrows (x, west to
// east) and j = 1..ncols (y, north to south) and is stored column-major,
// element (i, j) at [(j - 1) * nrows + (i - 1)]; cells are packed in that
// order over the mask.  Flow directions are mRM's codes as moveDownOneCell
// moves on this (i, j) grid (src/mRM/mo_mrm_net_startup.f90:1768-1801).
#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "network.h"

namespace mhm {

namespace {

constexpr int32_t kNodata = -9999;
constexpr double kDeltaH = 5.0; // floodplain elevation above the river bed [m], src/mRM/mo_mrm_constants.F90:38
constexpr double kEpsDp = 2.220446049250313e-16;

// moveDownOneCell, src/mRM/mo_mrm_net_startup.f90:1768-1801
void move_down(int32_t fdir, int32_t &i, int32_t &j)
{
    switch (fdir) {
    case 1: j += 1; break;
    case 2: i += 1; j += 1; break;
    case 4: i += 1; break;
    case 8: i += 1; j -= 1; break;
    case 16: j -= 1; break;
    case 32: i -= 1; j -= 1; break;
    case 64: i -= 1; break;
    case 128: i -= 1; j += 1; break;
    default: break; // sink
    }
}

// FORCES mo_utils le / ge (relative-epsilon comparisons)
bool le_dp(double a, double b) { return !(((kEpsDp * std::fabs(b) - std::fabs(a - b)) < 0.0) && (a > b)); }
bool ge_dp(double a, double b) { return !(((kEpsDp * std::fabs(b) - std::fabs(a - b)) < 0.0) && (a < b)); }

// 1-based 2-D grid accessor over a column-major array
template <class T>
struct Grid2 {
    std::vector<T> v;
    int32_t nr = 0, nc = 0;
    void init(int32_t r, int32_t c, T fill)
    {
        nr = r;
        nc = c;
        v.assign((size_t)r * c, fill);
    }
    T &operator()(int32_t i, int32_t j) { return v[(size_t)(j - 1) * nr + (i - 1)]; }
    bool in(int32_t i, int32_t j) const { return i >= 1 && i <= nr && j >= 1 && j <= nc; }
};

} // namespace

bool build_l11_network(const L0FlowInput &in, L11NetworkOut &out, std::string &err)
{
    const int32_t nr0 = in.nrows0, nc0 = in.ncols0, f = in.factor;
    if (nr0 < 1 || nc0 < 1 || f < 1) {
        err = "grid sizes and factor must be positive";
        return false;
    }
    // level-0 grid: ids, coordinates, flow data (unpack over the mask)
    Grid2<int32_t> id0, fdir0, facc0;
    Grid2<double> elev0;
    id0.init(nr0, nc0, kNodata);
    fdir0.init(nr0, nc0, kNodata);
    facc0.init(nr0, nc0, kNodata);
    elev0.init(nr0, nc0, -9999.0);
    std::vector<int32_t> ci0, cj0; // coordinates of packed L0 cell k (1-based)
    int32_t n0 = 0;
    for (int32_t j = 1; j <= nc0; ++j)
        for (int32_t i = 1; i <= nr0; ++i) {
            if (!in.mask0[(size_t)(j - 1) * nr0 + (i - 1)]) continue;
            id0(i, j) = n0 + 1;
            fdir0(i, j) = in.fdir0[n0];
            facc0(i, j) = in.facc0[n0];
            elev0(i, j) = in.elev0[n0];
            ci0.push_back(i);
            cj0.push_back(j);
            ++n0;
        }
    if (n0 != in.n_cells0) {
        err = "mask has " + std::to_string(n0) + " cells, expected " + std::to_string(in.n_cells0);
        return false;
    }
    // L11 grid over the L0 mask: init_lowres_level (src/common/mo_grid.f90:58-183)
    const int32_t nr11 = (nr0 + f - 1) / f, nc11 = (nc0 + f - 1) / f;
    Grid2<int32_t> mask11, id11;
    mask11.init(nr11, nc11, 0);
    id11.init(nr11, nc11, kNodata);
    for (int32_t j = 1; j <= nc0; ++j)
        for (int32_t i = 1; i <= nr0; ++i)
            if (id0(i, j) > 0) mask11((i + f - 1) / f, (j + f - 1) / f) = 1;
    std::vector<int32_t> ci11, cj11, iu, idn, jl, jr;
    Grid2<int32_t> l11_of0; // lowres_id_on_highres
    l11_of0.init(nr0, nc0, kNodata);
    int32_t L = 0;
    for (int32_t jc = 1; jc <= nc11; ++jc)
        for (int32_t ic = 1; ic <= nr11; ++ic) {
            if (!mask11(ic, jc)) continue;
            ++L;
            id11(ic, jc) = L;
            ci11.push_back(ic);
            cj11.push_back(jc);
            const int32_t u = (ic - 1) * f + 1, d = std::min(ic * f, nr0), l = (jc - 1) * f + 1,
                          r = std::min(jc * f, nc0);
            iu.push_back(u);
            idn.push_back(d);
            jl.push_back(l);
            jr.push_back(r);
            for (int32_t j = l; j <= r; ++j)
                for (int32_t i = u; i <= d; ++i) l11_of0(i, j) = L;
        }
    // L11_flow_direction (src/mRM/mo_mrm_net_startup.f90:227-629), the case of
    // fewer L11 than L0 cells
    Grid2<int32_t> fdir11, drasc0;
    fdir11.init(nr11, nc11, kNodata);
    drasc0.init(nr0, nc0, kNodata);
    std::vector<int32_t> row_out(L, kNodata), col_out(L, kNodata);
    std::vector<int32_t> oi, oj; // L0 outlet cells
    if (n0 == L) {
        err = "L11 resolution equal to L0 is not supported";
        return false;
    }
    for (int32_t k = 0; k < n0; ++k) {
        int32_t i = ci0[k], j = cj0[k];
        move_down(fdir0(i, j), i, j);
        const bool is_outlet = !fdir0.in(i, j) || fdir0(i, j) <= 0;
        if (!is_outlet) continue;
        oi.push_back(ci0[k]);
        oj.push_back(cj0[k]);
        const int32_t kk = l11_of0(ci0[k], cj0[k]);
        drasc0(ci0[k], cj0[k]) = kk;
        int32_t fmax = INT32_MIN;
        for (int32_t jj = jl[kk - 1]; jj <= jr[kk - 1]; ++jj)
            for (int32_t ii = iu[kk - 1]; ii <= idn[kk - 1]; ++ii) fmax = std::max(fmax, facc0(ii, jj));
        if (fmax == facc0(ci0[k], cj0[k])) {
            row_out[kk - 1] = ci0[k];
            col_out[kk - 1] = cj0[k];
            fdir11(ci11[kk - 1], cj11[kk - 1]) = 0;
        }
    }
    for (int32_t kk = 1; kk <= L; ++kk) {
        if (row_out[kk - 1] > 0) continue;
        const int32_t ic = ci11[kk - 1], jc = cj11[kk - 1];
        const int32_t u = iu[kk - 1], d = idn[kk - 1], l = jl[kk - 1], r = jr[kk - 1];
        int32_t fmax = -9, idmax = 0, side = -1;
        auto test = [&](int32_t i, int32_t j, int32_t a, int32_t b, int32_t c, int32_t s) {
            const int32_t fd = fdir0(i, j);
            if (facc0(i, j) > fmax && (fd == a || fd == b || fd == c)) {
                fmax = facc0(i, j);
                idmax = id0(i, j);
                side = s;
            }
        };
        for (int32_t jj = l; jj <= r; ++jj) test(u, jj, 32, 64, 128, 4);
        for (int32_t ii = u; ii <= d; ++ii) test(ii, r, 1, 2, 128, 1);
        for (int32_t jj = l; jj <= r; ++jj) test(d, jj, 2, 4, 8, 2);
        for (int32_t ii = u; ii <= d; ++ii) test(ii, l, 8, 16, 32, 3);
        if (idmax < 1) {
            err = "L11 cell " + std::to_string(kk) + " has no outflow across its border";
            return false;
        }
        const int32_t ii = ci0[idmax - 1], jj = cj0[idmax - 1];
        row_out[kk - 1] = ii;
        col_out[kk - 1] = jj;
        drasc0(ii, jj) = kk;
        const int32_t fd = fdir0(ii, jj);
        int32_t &o = fdir11(ic, jc);
        if (ii == u && jj == l) {
            if (fd == 8 || fd == 16) o = 16;
            else if (fd == 32) o = 32;
            else if (fd == 64 || fd == 128) o = 64;
        } else if (ii == u && jj == r) {
            if (fd == 32 || fd == 64) o = 64;
            else if (fd == 128) o = 128;
            else if (fd == 1 || fd == 2) o = 1;
        } else if (ii == d && jj == l) {
            if (fd == 2 || fd == 4) o = 4;
            else if (fd == 8) o = 8;
            else if (fd == 16 || fd == 32) o = 16;
        } else if (ii == d && jj == r) {
            if (fd == 128 || fd == 1) o = 1;
            else if (fd == 2) o = 2;
            else if (fd == 4 || fd == 8) o = 4;
        } else {
            o = side == 1 ? 1 : side == 2 ? 4 : side == 3 ? 16 : 64;
        }
    }
    int32_t n_out11 = 0;
    std::vector<int32_t> fd11(L), rows11(L), cols11(L);
    for (int32_t kk = 0; kk < L; ++kk) {
        fd11[kk] = fdir11(ci11[kk], cj11[kk]);
        rows11[kk] = ci11[kk];
        cols11[kk] = cj11[kk];
        if (fd11[kk] == 0) ++n_out11;
    }
    // links and routing order (L11_set_network_topology, L11_routing_order)
    std::vector<int32_t> from_n(L), to_n(L), perm(L), rord(L);
    int32_t n_links = 0;
    std::vector<int32_t> id2d((size_t)nr11 * nc11);
    for (int32_t jc = 1; jc <= nc11; ++jc)
        for (int32_t ic = 1; ic <= nr11; ++ic) id2d[(size_t)(jc - 1) * nr11 + (ic - 1)] = id11(ic, jc);
    if (!network_topology(nr11, nc11, id2d.data(), L, rows11.data(), cols11.data(), fd11.data(), from_n.data(),
                          to_n.data(), &n_links, err))
        return false;
    if (n_links != L - n_out11) {
        err = "links and outlets do not add up";
        return false;
    }
    if (L > 1 && !routing_order(L, n_out11, from_n.data(), to_n.data(), perm.data(), rord.data(), err)) return false;
    // L11_link_location (:887-1087): the first L0 cell of each link below its
    // from-node's outlet cell, and the L0 outlet cell it drains into
    std::vector<int32_t> f_row(L, kNodata), f_col(L, kNodata), t_row(L, kNodata), t_col(L, kNodata);
    for (int32_t rr = 0; rr < n_links; ++rr) {
        const int32_t ii = perm[rr] - 1;
        const int32_t node = from_n[ii];
        int32_t i = row_out[node - 1], j = col_out[node - 1];
        move_down(fdir0(i, j), i, j);
        f_row[ii] = i;
        f_col[ii] = j;
        bool is_outlet = false;
        for (size_t q = 0; q < oi.size(); ++q)
            if (i == oi[q] && j == oj[q]) is_outlet = true;
        if (!is_outlet) {
            while (!(drasc0.in(i, j) && drasc0(i, j) > 0)) {
                const int32_t pi = i, pj = j;
                if (!fdir0.in(i, j)) break;
                move_down(fdir0(i, j), i, j);
                if (pi == i && pj == j) {
                    err = "link location: the L0 flow path stops inside the basin";
                    return false;
                }
            }
        }
        t_row[ii] = i;
        t_col[ii] = j;
    }
    // L11_stream_features (:1233-1509): walk each link down its L0 river
    // cells; length (cartesian cell steps), slope over the walk (>= 1e-4) and
    // the floodplain: per river cell, the cells draining towards it within
    // deltaH above it (moveUp, :1595-1767, with its comparisons as written)
    Grid2<int32_t> fp0;
    fp0.init(nr0, nc0, kNodata);
    auto cell_length = [&](int32_t fd) {
        const double l = (fd == 2 || fd == 8 || fd == 32 || fd == 128) ? 1.4142135623730950488 : 1.0;
        return l * in.cellsize0; // iFlag_cordinate_sys = 0
    };
    std::vector<double> length(L, -9999.0), slope(L, -9999.0), afp(L, -9999.0);
    std::vector<std::vector<int32_t>> fp_cells(n_links);
    std::vector<int32_t> qi, qj; // the BFS queue (the reference's `stack`)
    for (int32_t rr = 0; rr < n_links; ++rr) {
        const int32_t ii = perm[rr] - 1, link = ii + 1;
        int32_t fr = f_row[ii], fc = f_col[ii];
        std::vector<int32_t> &mark = fp_cells[ii];
        auto set_fp = [&](int32_t i, int32_t j) {
            if (fp0(i, j) != link) mark.push_back(id0(i, j));
            fp0(i, j) = link;
        };
        set_fp(fr, fc);
        length[ii] = cell_length(fdir0(fr, fc));
        slope[ii] = elev0(fr, fc);
        int32_t fid = id0(fr, fc);
        const int32_t tid = id0(t_row[ii], t_col[ii]);
        while (fid != tid) {
            qi.assign(1, fr);
            qj.assign(1, fc);
            size_t head = 0;
            const double e0 = elev0(fr, fc);
            while (head < qi.size()) {
                const int32_t a = qi[head], b = qj[head];
                const int32_t ip = a + 1, im = a - 1, jp = b + 1, jm = b - 1;
                // the reference compares elev0(a, b + 1) in all but the first test
                const bool jp_ok = jp <= nc0;
                const double ej = jp_ok ? elev0(a, jp) : 0.0;
                auto push = [&](int32_t x, int32_t y, int32_t code, double ecmp) {
                    if (fdir0(x, y) == code && le_dp(elev0(x, y) - e0, kDeltaH) && ge_dp(ecmp - e0, 0.0)) {
                        qi.push_back(x);
                        qj.push_back(y);
                    }
                };
                if (jp_ok) push(a, jp, 16, elev0(a, jp));
                if (ip <= nr0 && jp_ok) push(ip, jp, 32, ej);
                if (ip <= nr0 && jp_ok) push(ip, b, 64, ej);
                if (ip <= nr0 && jp_ok && jm >= 1) push(ip, jm, 128, ej);
                if (jm >= 1 && jp_ok) push(a, jm, 1, ej);
                if (im >= 1 && jp_ok && jm >= 1) push(im, jm, 2, ej);
                if (im >= 1 && jp_ok) push(im, b, 4, ej);
                if (im >= 1 && jp_ok) push(im, jp, 8, ej);
                ++head;
                if (head < qi.size()) set_fp(qi[head], qj[head]);
            }
            move_down(fdir0(fr, fc), fr, fc);
            if (!fdir0.in(fr, fc) || id0(fr, fc) < 1) {
                err = "stream features: the river leaves the L0 mask";
                return false;
            }
            set_fp(fr, fc);
            fid = id0(fr, fc);
            length[ii] = length[ii] + cell_length(fdir0(fr, fc));
        }
        slope[ii] = (slope[ii] - elev0(fr, fc)) / length[ii];
        if (slope[ii] < 0.0001) slope[ii] = 0.0001;
        // the floodplain area: the cells marked for this link (a later link
        // may take some of them over, so sum now); cartesian cells have
        // equal areas, so the sum order does not matter
        double s = 0.0;
        for (size_t q = 0; q < mark.size(); ++q) s = s + in.cellsize0 * in.cellsize0;
        afp[ii] = s;
    }
    // L11_fraction_sealed_floodplain (:1510-1594): per land-cover scene, the
    // area of the link's final floodplain cells with the sealed class, over
    // the link's floodplain area
    std::vector<int32_t> fp_packed(n0, kNodata);
    for (int32_t k = 0; k < n0; ++k) fp_packed[k] = fp0(ci0[k], cj0[k]);
    out.frac_fp_imp.assign((size_t)in.n_lc_scenes * L, 0.0);
    for (int32_t sc = 0; sc < in.n_lc_scenes; ++sc) {
        const int32_t *lc = in.lcover0 + (size_t)sc * n0;
        std::vector<double> acc(n_links, 0.0);
        for (int32_t k = 0; k < n0; ++k) {
            const int32_t l = fp_packed[k];
            if (l >= 1 && l <= n_links && lc[k] == in.lc_class_imp) acc[l - 1] = acc[l - 1] + in.cellsize0 * in.cellsize0;
        }
        for (int32_t i = 0; i < n_links; ++i) out.frac_fp_imp[(size_t)sc * L + i] = acc[i] / afp[i];
    }
    out.n_nodes = L;
    out.n_outlets = n_out11;
    out.n_links = n_links;
    out.nrows11 = nr11;
    out.ncols11 = nc11;
    out.fdir11 = fd11;
    out.from_n = from_n;
    out.to_n = to_n;
    out.net_perm = perm;
    out.r_order = rord;
    out.length = length;
    out.slope = slope;
    out.a_floodplain = afp;
    out.row_out = row_out;
    out.col_out = col_out;
    out.cell_row11 = rows11;
    out.cell_col11 = cols11;
    out.n_l0_outlets = (int32_t)oi.size();
    return true;
}

// L11_L1_mapping (src/mRM/mo_mrm_net_startup.f90:61-226): the L1 and L11
// grids over the L0 mask at factors f1 and f11; every L1 cell gets the id of
// the L11 cell that contains it (L11 not finer than L1), or every L11 cell
// that of its L1 cell (L11 finer), -9999 otherwise.
bool l1_l11_mapping(int32_t nr0, int32_t nc0, const uint8_t *mask0, int32_t f1, int32_t f11,
                    std::vector<int32_t> &l1_l11, std::vector<int32_t> &l11_l1, std::string &err)
{
    if (nr0 < 1 || nc0 < 1 || f1 < 1 || f11 < 1 || (f11 % f1 != 0 && f1 % f11 != 0)) {
        err = "the L1 and L11 cell sizes must be integer multiples of each other";
        return false;
    }
    auto lowres = [&](int32_t f, Grid2<int32_t> &id, int32_t &n) {
        const int32_t nr = (nr0 + f - 1) / f, nc = (nc0 + f - 1) / f;
        Grid2<int32_t> m;
        m.init(nr, nc, 0);
        for (int32_t j = 1; j <= nc0; ++j)
            for (int32_t i = 1; i <= nr0; ++i)
                if (mask0[(size_t)(j - 1) * nr0 + (i - 1)]) m((i + f - 1) / f, (j + f - 1) / f) = 1;
        id.init(nr, nc, kNodata);
        n = 0;
        for (int32_t j = 1; j <= nc; ++j)
            for (int32_t i = 1; i <= nr; ++i)
                if (m(i, j)) id(i, j) = ++n;
    };
    Grid2<int32_t> id1, id11;
    int32_t n1 = 0, n11 = 0;
    lowres(f1, id1, n1);
    lowres(f11, id11, n11);
    Grid2<int32_t> on1, on11; // L11 id on the L1 grid, L1 id on the L11 grid
    on1.init(id1.nr, id1.nc, kNodata);
    on11.init(id11.nr, id11.nc, kNodata);
    if (f11 < f1) { // cellFactorRbyH < 1
        const int32_t inv = f1 / f11;
        for (int32_t jcc = 1; jcc <= id1.nc; ++jcc)
            for (int32_t icc = 1; icc <= id1.nr; ++icc) {
                if (id1(icc, jcc) < 1) continue;
                const int32_t u = (icc - 1) * inv + 1, d = std::min(icc * inv, id11.nr);
                const int32_t l = (jcc - 1) * inv + 1, r = std::min(jcc * inv, id11.nc);
                for (int32_t j = l; j <= r; ++j)
                    for (int32_t i = u; i <= d; ++i) on11(i, j) = id11(i, j) > 0 ? id1(icc, jcc) : kNodata;
            }
    } else {
        const int32_t fac = f11 / f1;
        for (int32_t jcc = 1; jcc <= id11.nc; ++jcc)
            for (int32_t icc = 1; icc <= id11.nr; ++icc) {
                if (id11(icc, jcc) < 1) continue;
                const int32_t u = std::max(1, (icc - 1) * fac + 1), d = std::min(icc * fac, id1.nr);
                const int32_t l = std::max(1, (jcc - 1) * fac + 1), r = std::min(jcc * fac, id1.nc);
                for (int32_t j = l; j <= r; ++j)
                    for (int32_t i = u; i <= d; ++i) on1(i, j) = id1(i, j) > 0 ? id11(icc, jcc) : kNodata;
            }
    }
    l1_l11.clear();
    l11_l1.clear();
    for (int32_t j = 1; j <= id1.nc; ++j)
        for (int32_t i = 1; i <= id1.nr; ++i)
            if (id1(i, j) > 0) l1_l11.push_back(on1(i, j));
    for (int32_t j = 1; j <= id11.nc; ++j)
        for (int32_t i = 1; i <= id11.nr; ++i)
            if (id11(i, j) > 0) l11_l1.push_back(on11(i, j));
    return true;
}

} // namespace mhm
