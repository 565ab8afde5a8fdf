// mpr_host.h -- parameter-independent start-up of the multiscale parameter
// regionalisation: soil horizon weights, empirical slope distribution,
// land-cover fractions and the L0 maps regrouped by L1 cell for the device.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "mhm_gpu.h"

namespace mhm {

// Packed per-L0-cell code, one 32-bit word per sub-cell slot:
//   bits  0-13  key = (soil id - 1) * 3 + (land cover - 1)
//   bit  14     northern hemisphere (y0 > 0)
//   bit  15     forest (land cover 1)
//   bits 16-23  LAI class - 1 (class-based LAI only)
//   bits 24-31  index of the nearest geological unit in GeoUnitList
constexpr int kMprKeyBits = 14;
constexpr uint32_t kMprKeyMask = (1u << kMprKeyBits) - 1u;
constexpr uint32_t kMprNorth = 1u << 14;
constexpr uint32_t kMprForest = 1u << 15;

struct MprSetup {
    int32_t n1 = 0, n0 = 0, max_sub = 0, H = 0;
    int32_t n_soil = 0, max_hor = 0, n_keys = 0, n_lai_classes = 0, n_geo = 0;
    int32_t n_lai_steps = 12;              // entries of the LAI input (12 for the look-up table)
    double dpth_t_last = 0.0;              // RZdepth of the soil of the last L0 cell
    std::vector<double> horizon_depth;     // [H], last entry = last soil type's RZdepth
    std::vector<double> Wd;                // [n_soil][H][max_hor]
    std::vector<double> slope_emp;         // [n0]
    std::vector<int32_t> nsub;             // [n1]
    std::vector<uint32_t> sub_code;        // [max_sub][n1]
    std::vector<double> sub_se, sub_asp;   // [max_sub][n1]
    std::vector<double> sub_lai;           // [n_lai_steps][max_sub][n1], gridded LAI only
    std::vector<double> f_forest, f_sealed, f_perm, f_kar; // [n1]
    std::vector<int32_t> n_hor, n_till, present; // [n_soil]
    std::vector<double> sand, clay, dbm;   // [n_soil][max_hor]
    std::vector<double> rz;                // [n_soil]
    std::vector<double> lai_lut;           // [n_lai_classes][12]
};

// generate_soil_database (src/MPR/mo_soil_database.f90:387-518), classical
// database: depth weights Wd[soil][horizon][soil layer].  horizon_depth[H-1]
// is overwritten with each soil type's RZdepth in turn, as the reference does.
bool soil_weights(int32_t n_soil, int32_t max_hor, const int32_t *n_hor, const double *ud, const double *ld,
                  const double *rz, int32_t H, double *horizon_depth, double *Wd, std::string &err);

// Empirical distribution of the L0 slope (L0_variable_init,
// src/MPR/mo_mpr_startup.f90:237-337).
void slope_empirical(int32_t n, const double *slope, double *slope_emp);

bool mpr_prepare(const mhm_l0_desc &l0, int32_t n1, int32_t H, MprSetup &out, std::string &err);

} // namespace mhm
