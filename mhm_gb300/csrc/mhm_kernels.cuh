// mhm_kernels.cuh -- shared declarations of the device kernels and their
// argument blocks (device layout of a context).
#pragma once
#include <cstdint>

namespace mhm {

constexpr int kMaxHorizons = 8;
constexpr int kForcKinds = 8; // pre, temp, pet, tmin, tmax, net radiation, abs. vapour pressure, wind speed

// Per-member effective-parameter planes, each [n_cells] contiguous:
// params[(m * n_planes + plane) * n_cells + k].
enum ParamPlane : int {
    P_FSEALED = 0,
    P_ALPHA,
    P_DDINC,
    P_DDMAX,
    P_DDNOPRE,
    P_FASP,
    P_HARSAM,
    P_KARST,
    P_K0, // kFastFlow
    P_K1, // kSlowFlow
    P_K2, // kBaseFlow
    P_KP, // kPerco
    P_JARVIS,
    P_TTHRESH,
    P_UTHRESH,
    P_STHRESH,
    P_MAXINTER,             // 12 planes (LAI month)
    P_PETLAI = P_MAXINTER + 12, // 12 planes: petLAIcorFactor, PrieTayAlpha or aeroResist (by PET case)
    P_PET2 = P_PETLAI + 12,     // 12 planes: surfResist (Penman-Monteith)
    P_HORIZON = P_PET2 + 12,    // then 5 groups of H planes: fRoots, SMs, FC, PW, beta
};
__host__ __device__ constexpr int n_param_planes(int H) { return P_HORIZON + 5 * H; }

// Per-member state planes: states[(m * n_planes + plane) * n_cells + k]
enum StatePlane : int { S_INTERC = 0, S_SNOW, S_SEAL, S_UNSAT, S_SAT, S_SM };
__host__ __device__ constexpr int n_state_planes(int H) { return S_SM + H; }

// One model step: forcing row (0-based within the device forcing window),
// calendar month (1..12), day flags and day of year.
enum StepFlags : int { SF_ISDAY = 1, SF_DAY_END = 2, SF_MONTH_END = 4, SF_YEAR_END = 8 };
struct StepInfo {
    int32_t row;
    int8_t month;
    int8_t dflags;  // SF_ISDAY: 6 < hour <= 18; SF_*_END: the next step starts a new day / month / year
    int16_t doy;
    int8_t hour;    // 0..23, the hour index of the meteo weights
    int16_t lai;    // iLAI: the month, or the index in a gridded LAI series (1-based)
};

// Aggregated flux/state outputs (outputFlxState of mhm_outputs.nml), indexes
// 1..21 of the reference's list; planes in the reference's write order.
constexpr int kOutFlags = 21;
enum OutFlag : int {
    OF_INTERC = 1, OF_SNOW, OF_SWC, OF_SM, OF_SM_ALL, OF_SEAL, OF_UNSAT, OF_SAT, OF_PET, OF_AET, OF_Q, OF_QD,
    OF_QIF, OF_QIS, OF_QB, OF_RECHARGE, OF_INFIL, OF_NEUTRONS, OF_AET_L, OF_PRE_EFFECT, OF_QSM
};
// Output of step tt (tindex = tt - warming steps > 0) closes an interval:
// src/common/mo_common_datetime_type.f90:157-185
__host__ __device__ inline bool out_writeout(int interval, int64_t tindex, int64_t tt, int64_t n_tt, int dflags)
{
    if (interval < -3) return false; // no output at all
    if (tt == n_tt) return true;     // the last step closes any open interval
    if (interval > 0) return tindex % interval == 0;
    if (interval == -1) return (dflags & SF_DAY_END) != 0;
    if (interval == -2) return (dflags & SF_MONTH_END) != 0;
    if (interval == -3) return (dflags & SF_YEAR_END) != 0;
    return false; // 0: only the last step
}

struct OutArgs {
    int32_t n_planes;        // 0: outputs off
    int32_t interval;        // timeStep_model_outputs
    int64_t warm_steps;      // no output for tt <= warm_steps
    int64_t n_tt;            // last step of the simulation period
    int64_t tt_base;         // absolute step of the chunk's step 0
    int32_t slot0, cnt0;     // slots written before this chunk, steps in the open interval
    int32_t max_slots;       // slots of `out` (writes past it are dropped; the host refuses such runs)
    int8_t plane[kOutFlags + 1]; // first plane of flag f (1-based), -1 if off
    uint64_t avg_mask;       // planes written as a mean over the interval (states)
    double *acc;             // [n_planes][M][n_cells] running sums
    double *out;             // [slots][n_planes][M][n_cells]
    // outputs of step tt_w[m] weighted with these fSealed / soilMoistSat
    // instead of the member's parameters (the next land-cover scene's)
    const int64_t *tt_w;     // [M]
    const double *w_fsealed; // [M][n_cells]
    const double *w_sms;     // [M][H][n_cells]
};

struct MonthTables {
    double evap[12];
    double fday_prec[12], fnight_prec[12];
    double fday_pet[12], fnight_pet[12];
    double fday_temp[12], fnight_temp[12];
};

struct CellArgs {
    int32_t n_cells, n_members, n_steps;
    int32_t proc_sm, proc_pet, is_hourly;
    int32_t reset_sm;   // tt == 1 && !read_states: SM = 0.5 * FC before the first step
    int32_t row_base;   // forcing row (1-based iMeteoTS) stored first in the buffers
    double c2TSTu;      // timestep / 24
    double nTstepDay;   // 24 / timestep
    const double *pre, *temp, *pet, *tmin, *tmax; // [rows][n_cells] from row_base
    const double *netrad;                         // [rows][n_cells] (proc_pet 2, 3) or null
    const double *eabs, *wind;                    // [rows][n_cells] (proc_pet 3) or null
    // read_meteo_weights: L1_{pre,pet,temp}_weights(cell, month, hour) as
    // [24][12][n_cells] (the reference's column-major order); null: day/night ratios
    const double *w_pre, *w_pet, *w_temp;
    const StepInfo *steps;                        // [n_steps]
    const double *params;                         // [M][planes][n_cells]
    double *states;                               // [M][planes][n_cells]
    double *tro;                                  // [n_steps][M][n_cells]
    const double *latitude;                       // [n_cells]
    MonthTables tab;
    // member mode (each member at its own model step; hourly, device forcing
    // window shared by all members): member m's step t of this chunk is
    // steps[member_step0[m] + step_shift + t] and reads window row
    // step_shift + t; member_step0[m] < 0 marks an idle member (no work,
    // zero runoff).  member_step0 == nullptr: all members at the same step.
    const int32_t *member_step0;
    int32_t step_shift;
    int32_t reset_ok;   // member mode: SM = 0.5 * FC when a member is at its step 1
    // optional per-step fluxes [n_steps][M][n_cells] (nullptr = off): total
    // actual ET (canopy + sealed + soil, area weighted) and the percolation
    // lost to (or, karstLoss > 1, gained from) outside the cell
    double *flux_aet, *flux_loss;
    OutArgs out;        // aggregated flux/state outputs (flux variant only)
    // per-member failure flag: bit 0 set when the member's total runoff of a
    // step or a state at the chunk's end is not finite (nullptr = not checked)
    int32_t *nonfinite;
    int32_t n_horizons; // the context's horizon count (read by the fused multi-context launch)
    // extents the bounds-checked build tests its data-derived indexes against:
    // forcing rows from row_base (or window rows in member mode) and, in member
    // mode, the rows of the member step table
    int32_t n_forc_rows, n_step_rows;
    // gridded LAI series (timeStep_LAI_input -1 / -2 / -3): the LAI-indexed
    // parameters as [M][lai_groups(proc_pet)][n_lai][n_cells] -- maxInter,
    // then the petLAIcorFactor / PrieTayAlpha / aeroResist group and
    // surfResist where the PET case reads them -- read at step.lai instead of
    // the monthly planes; nullptr: monthly slots
    const double *lai_series;
    int32_t n_lai;
};

// LAI-indexed parameter groups a gridded LAI series holds for a PET case:
// maxInter always; the LAI correction factor (-1), Priestley-Taylor alpha (2)
// or aerodynamic resistance (3); the bulk surface resistance (3)
__host__ __device__ constexpr int lai_groups(int proc_pet)
{
    return 1 + ((proc_pet == -1 || proc_pet >= 2) ? 1 : 0) + (proc_pet == 3 ? 1 : 0);
}

// One persistent launch of the cell chain over several contexts (with the
// same process cases' code path): tile t covers work items
// tile_item0[t] .. + 127 of context tile_ctx[t].
struct FusedCellArgs {
    const CellArgs *args;       // [n_contexts]
    const int32_t *tile_ctx;    // [n_tiles]
    const int64_t *tile_item0;  // [n_tiles]
    int32_t n_tiles;
    int32_t *queue;             // next tile to take (0 before the launch)
};

struct AccArgs {
    int32_t n_cells, n_nodes, n_members, n_steps;   // n_steps: routing steps written to qout
    int32_t map_flag;
    int32_t win;                 // model steps summed per routing step (adaptive routing, else 1)
    double TST;                  // HourSecs * routing timestep
    const double *tro;           // [n_steps][M][n_cells]
    const double *l1_area;       // [n_cells]
    const int32_t *node_cell_ptr; // [n_nodes+1] by level position
    const int32_t *node_cells;    // ascending L1 index per node
    const int32_t *pos_l11_l1;    // [n_nodes] 0-based L1 cell of the node (!map_flag)
    const double *pos_area;       // [n_nodes] L11 area by position
    double *qout;                 // [M][n_steps][n_nodes] by level position
    const int32_t *member_step0;  // member mode: < 0 marks an idle member (skipped)
};

// Wavefront routing: the chunk is cut into sub-chunks of `sub` steps; launch
// `tick` advances sub-chunk (tick - level) of every node whose level is in
// [lvl_lo, lvl_hi] (positions pos_begin .. pos_end-1).
struct RouteArgs {
    int32_t n_nodes, n_members, n_steps;
    int32_t pos_begin, pos_end;
    int32_t tick, sub;
    const int32_t *pos_level;   // [n_nodes] topological level of each position
    const int32_t *up_ptr;      // [n_nodes+1]
    const int32_t *up_pos;      // upstream positions in rank order
    const int8_t *pos_flags;    // bit0: is link (has C1/C2), bit1: add qOUT, bit2: the link's routed
                                // outflow is cut (it drains into a non-headwater inflow gauge's node)
    const double *C1, *C2;      // [M][n_nodes] by position
    // routing step s reads qOUT row s / rdiv of [M][n_qsteps][n_nodes]: with an
    // adaptive routing step shorter than the model step the model step's qOUT
    // is routed rdiv times
    int32_t rdiv, n_qsteps;
    const double *qout;
    double *qtr;                // [M][n_steps][n_nodes] routed outflow series
    double *qmod;               // [M][n_steps][n_nodes] (if write_qmod)
    double *qtin1, *qtr1;       // [M][n_nodes] state (previous step)
    const int32_t *member_step0; // member mode: < 0 marks an idle member (skipped)
};

// The wavefront of a chunk walked in one launch (route_walk_kernel): tick k
// spans levels max(0, k - n_sub + 1) .. min(k, n_levels - 1), i.e. positions
// level_ptr[lo] .. level_ptr[hi + 1] - 1.
struct RouteWalk {
    const int32_t *level_ptr; // [n_levels + 1] first routing position of each level
    int32_t n_levels, n_sub, n_ticks;
};

// add_inflow (src/mRM/mo_mrm_pre_routing.f90:179-214) on a chunk's qOUT rows,
// after the L1->L11 accumulation: per (member, routing step) the inflow
// gauges in list order add their discharge to (headwater) or put it in place
// of the node's runoff.  The discharge of a model step is the gauge's value
// of day ceiling(tt / steps_day) (iDischargeTS); with `mean` (adaptive
// routing whose routing step is not shorter than the model step) it is the
// sum over the routing step's `win` model steps from 0, divided by tsf
// (tsRoutFactorIn), src/mHM/mo_mhm_interface_run.f90:463-511.
constexpr int kMaxInflow = 64;
struct InflowArgs {
    int32_t n_members, n_qsteps, n_nodes, n_inflow;
    int32_t win, steps_day, day0, mean;
    double tsf;
    int64_t tt_base;             // model step (1-based) of the chunk's first step
    const int32_t *member_step0; // member mode: member m's chunk step t is tt = member_step0[m] + step_shift + t + 1
    int32_t step_shift;
    const int32_t *pos;          // [n_inflow] routing position of each gauge's node
    const int8_t *headwater;     // [n_inflow]
    const double *q;             // [days][n_inflow] from day0
    int32_t n_days;              // rows of q
    double *qout;                // [M][n_qsteps][n_nodes]
};

// Per-model-step L11 discharge from the routing steps (adaptive routing):
// rdiv > 1: the mean of the step's rdiv routing passes, ((0 + Q_1) + Q_2 ...)
// / rdiv (src/mRM/mo_mrm_routing.f90:238-277); win > 1: the routing step's
// value for each of its win model steps (src/mHM/mo_mhm_interface_run.f90:603-608)
struct QmodStepArgs {
    int32_t n_members, n_steps, n_nodes, rdiv, win;
    const double *qmod_sub;     // [M][n_steps * rdiv / win][n_nodes]
    double *qmod;               // [M][n_steps][n_nodes]
    const int32_t *member_step0;
};

// mRM's Qrouted output: per model step the L11 discharge state (with a routing
// step of `win` model steps it changes only at the last step of each window),
// aggregated as a mean over the output interval
// (src/mRM/mo_mrm_write_fluxes_states.f90:130-133, src/common/mo_nc_output.f90:140-175)
struct QroutArgs {
    int32_t n_members, n_steps, n_nodes, win, interval;
    int32_t slot0, cnt0, max_slots;
    int64_t warm_steps, n_tt, tt_base;
    int32_t jul_start, timestep; // calendar (interval ends)
    const double *qmod;          // [M][n_steps][n_nodes]
    const double *qmod_prev;     // [M][n_nodes] discharge state before the chunk
    double *acc;                 // [M][n_nodes]
    double *out;                 // [slots][M][n_nodes]
};

struct GaugeArgs {
    int32_t n_members, n_steps, n_nodes, n_gauges;
    int32_t step_offset, total_steps;
    const int32_t *gauge_pos;
    const double *qmod;    // [M][n_steps][n_nodes]
    double *q_gauge;       // [M][n_gauges][total_steps]
    const int32_t *member_step0; // member mode: idle members get zero discharge
};

// ---- multiscale parameter regionalisation ----
constexpr int kMprMaxSoilHor = 16;
// entries of one (soil, land cover) row of the per-member soil table
__host__ __device__ constexpr int mpr_table_stride(int H) { return 5 * H + 4; }
enum MprTableCol : int { MT_INV_SMS = 0, MT_INV_BETA = 1, MT_INV_PW = 2, MT_INV_FC = 3, MT_INV_FROOTS = 4 };

// start of each process's block in the global parameter vector
struct GammaOffsets {
    int32_t interc, snow, soil, runoff, pet, interflow, perc, routing, geo, total;
    int32_t n_soil_params;
};

struct MprArgs {
    int32_t n1, max_sub, H, proc_sm, proc_pet;
    int32_t n_soil, max_hor, n_keys, n_lai_classes, n_gamma, n_members;
    GammaOffsets off;
    double dpth_t_last;            // RZdepth of the last L0 cell's soil
    // soil database [n_soil] / [n_soil][max_hor] / Wd [n_soil][H][max_hor]
    const int32_t *n_hor, *n_till;
    const double *sand, *clay, *dbm, *rz, *Wd, *hd;
    const double *lai_lut;         // [n_lai][12]
    // L0 sub-cells of every L1 cell, slot-major [max_sub][n1]
    const int32_t *nsub;           // [n1]
    const uint32_t *code;
    const double *se, *asp;
    const double *lai;             // [12][max_sub][n1] gridded LAI or null
    const double *f_forest, *f_sealed, *f_perm, *f_kar; // [n1]
    const double *gamma;           // [n_members][n_gamma]
    double *table;                 // [n_members][n_keys][stride]
    double *petlai;                // [n_members][3][n_lai][12] reciprocal factors
    double *params;                // effective parameters of the first member
    int64_t member_stride;         // doubles between members' parameter blocks
    // LAI entries (12 monthly slots, or a gridded series) and, for a series,
    // where its LAI-indexed parameters go: [member][3][n_lai_steps][n1] from
    // the first member's block (maxInter, petLAIcorFactor / PrieTayAlpha /
    // aeroResist, surfResist); nullptr: the monthly parameter planes
    int32_t n_lai_steps;
    double *lai_out;
};


} // namespace mhm
