// network.h -- host-side preparation of an L11 routing network for the
// level-synchronous device routing, and the model-step calendar.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace mhm {

// Routing network laid out by topological level (positions 0..n_nodes-1).
struct LevelNetwork {
    int32_t n_nodes = 0, n_links = 0, n_levels = 0;
    std::vector<int32_t> level_ptr;  // [n_levels + 1] position ranges
    std::vector<int32_t> pos_of_node; // [n_nodes] 0-based node -> position
    std::vector<int32_t> node_of_pos; // [n_nodes]
    std::vector<int32_t> up_ptr;      // [n_nodes + 1] by position
    std::vector<int32_t> up_pos;      // upstream positions, netPerm rank order
    std::vector<int8_t> pos_flags;    // bit0 is link, bit1 adds its own qOUT
    std::vector<int32_t> link_pos;    // [n_links] 1-based link i-1 -> position of fromN(i)
    int32_t max_width = 0;
};

// Builds the level layout from L11_netPerm / L11_fromN / L11_toN (1-based, as
// produced by L11_set_network_topology and L11_routing_order,
// src/mRM/mo_mrm_net_startup.f90:630-886).  Fails (returns false, message in
// err) unless netPerm is a permutation of the links in which every link comes
// after all links that drain into its source node -- the order the reference
// routes in (src/mRM/mo_mrm_routing.f90:435-459).
bool build_level_network(int32_t n_nodes, int32_t n_outlets, const int32_t *net_perm, const int32_t *from_n,
                         const int32_t *to_n, LevelNetwork &out, std::string &err);

// Routing order of L11_routing_order (src/mRM/mo_mrm_net_startup.f90:728-886)
// computed with per-link counts of unranked upstream links instead of the
// reference's all-pairs scan: O(n_links x sweeps).  Same ranks, same netPerm.
bool routing_order(int32_t n_nodes, int32_t n_outlets, const int32_t *from_n, const int32_t *to_n,
                   int32_t *net_perm, int32_t *r_order, std::string &err);

// L11 links from the L11 flow directions (L11_set_network_topology,
// src/mRM/mo_mrm_net_startup.f90:630-727): cell k (1-based, packed order)
// drains into the cell its D8 code points at; cells pointing at themselves
// (outlets) give no link.  id2d [ncols][nrows] holds the 1-based cell id of
// every grid cell (column-major over (row, col)); from_n / to_n [n_cells]
// receive the links in cell order, -9999 past the last.
bool network_topology(int32_t nrows, int32_t ncols, const int32_t *id2d, int32_t n_cells, const int32_t *cell_row,
                      const int32_t *cell_col, const int32_t *fdir, int32_t *from_n, int32_t *to_n, int32_t *n_links,
                      std::string &err);

// Level-0 flow data of one basin for mRM's network start-up.
struct L0FlowInput {
    int32_t nrows0 = 0, ncols0 = 0; // L0 grid (mHM's (x, y) order, column-major)
    int32_t factor = 0;             // L11 cell size / L0 cell size
    int32_t n_cells0 = 0;           // cells of the mask
    const uint8_t *mask0 = nullptr; // [ncols0][nrows0]
    const int32_t *fdir0 = nullptr, *facc0 = nullptr; // [n_cells0] packed over the mask
    const double *elev0 = nullptr;  // [n_cells0]
    double cellsize0 = 0.0;         // [m], cartesian coordinates
    int32_t n_lc_scenes = 0, lc_class_imp = 2;
    const int32_t *lcover0 = nullptr; // [n_lc_scenes][n_cells0]
};

// The L11 network mRM derives from it (arrays over the L11 cells; link
// arrays valid for 1..n_links).
struct L11NetworkOut {
    int32_t n_nodes = 0, n_outlets = 0, n_links = 0, nrows11 = 0, ncols11 = 0, n_l0_outlets = 0;
    std::vector<int32_t> fdir11, cell_row11, cell_col11, from_n, to_n, net_perm, r_order, row_out, col_out;
    std::vector<double> length, slope, a_floodplain;
    std::vector<double> frac_fp_imp; // [n_lc_scenes][n_nodes]
};

// L11_flow_direction, L11_set_network_topology, L11_routing_order,
// L11_link_location, L11_stream_features and L11_fraction_sealed_floodplain
// (src/mRM/mo_mrm_net_startup.f90:227-1594) for an L11 grid coarser than L0,
// cartesian coordinates (iFlag_cordinate_sys = 0).
bool build_l11_network(const L0FlowInput &in, L11NetworkOut &out, std::string &err);

// L11_L1_mapping (src/mRM/mo_mrm_net_startup.f90:61-226) for L1 and L11
// grids at factors f1 and f11 of the L0 grid: L1_L11_Id [L1 cells] and
// L11_L1_Id [L11 cells].
bool l1_l11_mapping(int32_t nr0, int32_t nc0, const uint8_t *mask0, int32_t f1, int32_t f11,
                    std::vector<int32_t> &l1_l11, std::vector<int32_t> &l11_l1, std::string &err);

} // namespace mhm
