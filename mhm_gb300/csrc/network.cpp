// network.cpp -- routing-level layout and routing order (host).
#include "network.h"

#include <algorithm>
#include <numeric>

namespace mhm {

bool build_level_network(int32_t L, int32_t n_outlets, const int32_t *net_perm, const int32_t *from_n,
                         const int32_t *to_n, LevelNetwork &o, std::string &err)
{
    o = LevelNetwork{};
    if (L < 1 || n_outlets < 1 || n_outlets > L) {
        err = "network: need n_nodes >= 1 and 1 <= n_outlets <= n_nodes";
        return false;
    }
    const int32_t nl = L - n_outlets;
    o.n_nodes = L;
    o.n_links = nl;
    std::vector<int32_t> rank(nl, -1), out_link(L, -1);
    for (int32_t r = 0; r < nl; ++r) {
        const int32_t i = net_perm[r] - 1;
        if (i < 0 || i >= nl || rank[i] != -1) {
            err = "network: netPerm is not a permutation of the links";
            return false;
        }
        rank[i] = r;
    }
    for (int32_t i = 0; i < nl; ++i) {
        const int32_t f = from_n[i] - 1, t = to_n[i] - 1;
        if (f < 0 || f >= L || t < 0 || t >= L || f == t) {
            err = "network: fromN/toN out of range or self loop";
            return false;
        }
        if (out_link[f] != -1) {
            err = "network: a node is the source of two links";
            return false;
        }
        out_link[f] = i;
    }
    // upstream links per node, in rank order
    std::vector<std::vector<int32_t>> ups(L);
    for (int32_t r = 0; r < nl; ++r) {
        const int32_t i = net_perm[r] - 1;
        ups[to_n[i] - 1].push_back(i);
    }
    // topological check: every upstream link of fromN(i) precedes i
    for (int32_t i = 0; i < nl; ++i)
        for (int32_t j : ups[from_n[i] - 1])
            if (rank[j] >= rank[i]) {
                err = "network: netPerm is not a topological order of the links";
                return false;
            }
    // levels (longest path from a headwater), relaxed in rank order
    std::vector<int32_t> level(L, 0);
    for (int32_t r = 0; r < nl; ++r) {
        const int32_t i = net_perm[r] - 1;
        const int32_t f = from_n[i] - 1, t = to_n[i] - 1;
        level[t] = std::max(level[t], level[f] + 1);
    }
    const int32_t special_outlet = (nl > 0) ? to_n[net_perm[nl - 1] - 1] - 1 : -1;
    // positions: by level, then by rank of the node's link (sinks last)
    std::vector<int32_t> order(L);
    std::iota(order.begin(), order.end(), 0);
    auto key = [&](int32_t v) { return out_link[v] >= 0 ? (int64_t)rank[out_link[v]] : (int64_t)nl + v; };
    std::stable_sort(order.begin(), order.end(), [&](int32_t a, int32_t b) {
        if (level[a] != level[b]) return level[a] < level[b];
        return key(a) < key(b);
    });
    o.node_of_pos = order;
    o.pos_of_node.assign(L, 0);
    for (int32_t p = 0; p < L; ++p) o.pos_of_node[order[p]] = p;
    o.n_levels = level[order[L - 1]] + 1;
    o.level_ptr.assign(o.n_levels + 1, 0);
    for (int32_t v = 0; v < L; ++v) o.level_ptr[level[v] + 1]++;
    for (int32_t l = 0; l < o.n_levels; ++l) o.level_ptr[l + 1] += o.level_ptr[l];
    for (int32_t l = 0; l < o.n_levels; ++l)
        o.max_width = std::max(o.max_width, o.level_ptr[l + 1] - o.level_ptr[l]);
    o.up_ptr.assign(L + 1, 0);
    o.pos_flags.assign(L, 0);
    for (int32_t p = 0; p < L; ++p) {
        const int32_t v = order[p];
        o.up_ptr[p + 1] = o.up_ptr[p] + (int32_t)ups[v].size();
        for (int32_t j : ups[v]) o.up_pos.push_back(o.pos_of_node[from_n[j] - 1]);
        int8_t fl = 0;
        if (out_link[v] >= 0) fl |= 3; // a link adds its own qOUT (mo_mrm_routing.f90:445)
        if (v == special_outlet) fl |= 2; // mo_mrm_routing.f90:466-467
        o.pos_flags[p] = fl;
    }
    o.link_pos.assign(nl, 0);
    for (int32_t i = 0; i < nl; ++i) o.link_pos[i] = o.pos_of_node[from_n[i] - 1];
    return true;
}

bool routing_order(int32_t L, int32_t n_outlets, const int32_t *from_n, const int32_t *to_n, int32_t *net_perm,
                   int32_t *r_order, std::string &err)
{
    const int32_t nl = L - n_outlets;
    for (int32_t i = 0; i < L; ++i) net_perm[i] = r_order[i] = -9999;
    if (L <= 1) return true;
    if (nl < 0) {
        err = "routing_order: n_outlets > n_nodes";
        return false;
    }
    // pending[i]: number of unranked links draining into fromN(i) (self excluded,
    // as in the reference's jj == ii test).
    std::vector<int32_t> pending(nl, 0);
    std::vector<std::vector<int32_t>> into(L); // links whose toN is node v
    for (int32_t j = 0; j < nl; ++j) {
        const int32_t t = to_n[j] - 1;
        if (t < 0 || t >= L) {
            err = "routing_order: toN out of range";
            return false;
        }
        into[t].push_back(j);
    }
    std::vector<std::vector<int32_t>> feeds(nl); // feeds[j]: links i with fromN(i) == toN(j)
    for (int32_t i = 0; i < nl; ++i) {
        const int32_t f = from_n[i] - 1;
        if (f < 0 || f >= L) {
            err = "routing_order: fromN out of range";
            return false;
        }
        for (int32_t j : into[f])
            if (j != i) {
                pending[i]++;
                feeds[j].push_back(i);
            }
    }
    std::vector<int32_t> rank(nl, 0);
    int32_t kk = 0;
    std::vector<int32_t> unranked;
    for (int32_t i = 0; i < nl; ++i) {
        if (pending[i] == 0) {
            rank[i] = ++kk; // headwaters in link order
        } else {
            unranked.push_back(i);
        }
    }
    for (int32_t i = 0; i < nl; ++i)
        if (rank[i] > 0)
            for (int32_t d : feeds[i]) pending[d]--;
    // sweeps in link order; a link ranked earlier in the same sweep counts
    while (!unranked.empty()) {
        std::vector<int32_t> rest;
        bool progress = false;
        for (int32_t i : unranked) {
            if (pending[i] == 0) {
                rank[i] = ++kk;
                progress = true;
                for (int32_t d : feeds[i]) pending[d]--;
            } else {
                rest.push_back(i);
            }
        }
        if (!progress) {
            err = "routing_order: network has a cycle";
            return false;
        }
        unranked.swap(rest);
    }
    for (int32_t i = 0; i < nl; ++i) {
        r_order[i] = rank[i];
        net_perm[rank[i] - 1] = i + 1;
    }
    return true;
}

bool network_topology(int32_t nrows, int32_t ncols, const int32_t *id2d, int32_t n_cells, const int32_t *cell_row,
                      const int32_t *cell_col, const int32_t *fdir, int32_t *from_n, int32_t *to_n, int32_t *n_links,
                      std::string &err)
{
    for (int32_t k = 0; k < n_cells; ++k) from_n[k] = to_n[k] = -9999; // nodata_i4
    int32_t nl = 0;
    for (int32_t k = 0; k < n_cells; ++k) {
        // row / column offsets of the ESRI D8 codes, as moveDownOneCell
        // steps them (src/mRM/mo_mrm_net_startup.f90:1768-1801); any other
        // code leaves the cell where it is
        int32_t di = 0, dj = 0;
        switch (fdir[k]) {
        case 1: dj = 1; break;
        case 2: di = 1; dj = 1; break;
        case 4: di = 1; break;
        case 8: di = 1; dj = -1; break;
        case 16: dj = -1; break;
        case 32: di = -1; dj = -1; break;
        case 64: di = -1; break;
        case 128: di = -1; dj = 1; break;
        default: break;
        }
        const int32_t i = cell_row[k] + di, j = cell_col[k] + dj; // 1-based
        if (i < 1 || i > nrows || j < 1 || j > ncols) {
            err = "network_topology: flow direction of cell " + std::to_string(k + 1) + " leaves the grid";
            return false;
        }
        const int32_t to = id2d[(size_t)(j - 1) * nrows + (i - 1)];
        if (to == k + 1) continue; // points at itself: an outlet
        if (to < 1 || to > n_cells) {
            err = "network_topology: flow direction of cell " + std::to_string(k + 1) + " leaves the mask";
            return false;
        }
        from_n[nl] = k + 1;
        to_n[nl] = to;
        ++nl;
    }
    *n_links = nl;
    return true;
}

} // namespace mhm
