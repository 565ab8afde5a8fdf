// cell_chain_impl.cuh -- the mHM L1 cell chain as one time-looping kernel
// (included by the translation units that instantiate its register/occupancy
// variants).
//
// One thread advances one (member, cell) through a chunk of time steps with
// all states and effective parameters in registers; forcing is read once per
// step as coalesced [step][cell] rows and the step's total runoff is written
// as a coalesced [step][member][cell] row.  The arithmetic of every step is
// the reference's, in the reference's order (compiled with --fmad=false;
// log/exp/pow from hmath.h), so a step here equals a step of
//   mHM() cell loop              src/mHM/mo_mhm.f90:458-517
//   get_corrected_pet/temp/prec  src/meteo/mo_meteo_handler.f90:915-1285
// bit for bit.  Expressions that depend on parameters only (c2TSTu/k, the
// degree-day threshold, FC-PW, ...) are evaluated once per chunk: the same
// operands give the same bits as the reference's per-step evaluation.
#pragma once
#include <cfloat>
#include <cmath>

#include "bounds.cuh"
#include "calendar.h"
#include "fp64i.h"
#include "hmath.h"
#include "mhm_kernels.cuh"

namespace mhm {

namespace {

constexpr double kEps = DBL_EPSILON; // src/common/mo_common_constants.f90:25
constexpr double kTwoThird = 2.0 / 3.0;
constexpr double kPiD = 3.141592653589793238462643383279502884197;
constexpr double kTwoPiD = 6.283185307179586476925286766559005768394;
constexpr double kDaySecs = 86400.0, kYearDays = 365.0, kSolarConst = 1367.0, kSpecHeatET = 2.45e06;
constexpr double kDeg2Rad = 3.141592653589793238462643383279502884197 / 180.0;
constexpr double kHarSamConst = 17.800;
// src/common/mo_constants.f90 (Psychro_dp) and src/mHM/mo_mhm_constants.f90 (tetens_c*, satpressureslope1)
constexpr double kPsychro = 0.0646, kTetensC1 = 0.6108, kTetensC2 = 17.270, kTetensC3 = 237.30;
constexpr double kSatPressureSlope1 = 4098.0;
constexpr double kT0 = 273.15; // FORCES mo_constants T0_dp (Celsius <-> Kelvin)
constexpr double kRho0 = 1.225, kCp0 = 1005.0; // air density, heat capacity (FORCES mo_constants)

// src/mHM/mo_pet.f90:314-355 (CUDA's sin/cos/tan/acos; only the daily-forcing
// Hargreaves variant uses it)
__device__ double extraterr_rad_approx(int doy, double latitude)
{
    double dr = 1.0 + 0.0330 * cos(kTwoPiD * doy / kYearDays);
    double delta = 0.4090 * sin(kTwoPiD * doy / kYearDays - 1.3900);
    double arg = -tan(latitude) * tan(delta);
    if (arg < -1.0) arg = -1.0;
    if (arg > 1.0) arg = 1.0;
    double omega = acos(arg);
    return kDaySecs / kPiD / kSpecHeatET * kSolarConst * dr *
           (omega * sin(latitude) * sin(delta) + cos(latitude) * cos(delta) * sin(omega));
}

// FORCES mo_utils LE (in-tree copy pre-proc/mtCLIM/mo_utils.f90 lesserequal_dp)
__device__ __forceinline__ bool le_dp(double a, double b)
{
    return !(((kEps * fabs(b) - fabs(a - b)) < 0.0) && (a > b));
}

// src/mHM/mo_pet.f90:73-116
__device__ double pet_hargreaves(double coeff, double tavg, double tmax, double tmin, double rad)
{
    double delta_temp = tmax - tmin;
    if (le_dp(delta_temp, 0.0) || le_dp(tavg, -kHarSamConst)) return 0.0;
    return coeff * rad * (tavg + kHarSamConst) * sqrt(delta_temp);
}

// src/mHM/mo_pet.f90:149-174 (pet_priestly), with slope_satpressure (:384-399)
// and sat_vap_pressure written as the reference does: exp(2 log(T + c3)) for
// the square, divisions in the same order
__device__ double pet_priestly(double alpha, double rn, double tavg)
{
    const double svp = kTetensC1 * hm_exp(kTetensC2 * tavg / (tavg + kTetensC3));
    const double delta = kSatPressureSlope1 * svp / hm_exp(2.0 * hm_log(tavg + kTetensC3));
    return alpha * delta / (kPsychro + delta) * (rn * kDaySecs / kSpecHeatET);
}

// src/mHM/mo_pet.f90:235-272 (pet_penman) with a_s = a_sh = 1, as the meteo
// handler calls it (mo_meteo_handler.f90:1087-1095); the same operation order
__device__ double pet_penman(double net_rad, double tavg, double act_vap, double ra, double rs)
{
    const double svp = kTetensC1 * hm_exp(kTetensC2 * tavg / (tavg + kTetensC3));
    const double slope = kSatPressureSlope1 * svp / hm_exp(2.0 * hm_log(tavg + kTetensC3));
    return kDaySecs / kSpecHeatET * (slope * net_rad + kRho0 * kCp0 * (svp - act_vap) * 1.0 / ra) /
           (slope + kPsychro * 1.0 / 1.0 * (1.0 + rs / ra));
}

// Per-thread scalars live in registers; the soil moisture of each horizon
// and two reciprocals per horizon live in shared memory, [plane][H][blockDim]
// (consecutive threads -> consecutive words), so the horizon loop stays
// rolled: fewer registers (more warps per SM) and a smaller instruction
// footprint.
struct CellRegs {
    // states
    double interc, snow, seal, unsat, sat;
    // parameters (and parameter-only derived values)
    double fsealed, fnotsealed; // fnotsealed = 1 - fsealed (parameter only)
    double ddinc, ddmax_s, ddnopre_s, dd_thr;
    double tthresh, sthresh, uthresh, karst, alpha1;
    double k0s, k1s, k2s, kps; // c2TSTu / k
    double jarvis;
    double fasp, harsam, lat_rad;
    uint64_t r_sthresh, r_jarvis; // reciprocals of the chunk-fixed divisors
};
// Every division of the step divides by a value that is fixed over the chunk
// (SMs, the stress denominator FC - PW or SMs - PW, sealedThresh, the Jarvis
// threshold) or over a month (interception capacity, pan-evaporation
// coefficient): their fixed-point reciprocals (hm_recip_of) are computed once
// and each division runs hm_div_r -- the same correctly rounded quotient as
// hm_div at about half its integer instructions.  HS_RSMS / HS_RDEN hold the
// reciprocals' bits.
//
// The read-only per-horizon parameters (fRoots, SMs, FC, PW, beta) are copied
// to shared memory too when that costs no occupancy -- up to 3 horizons,
// where 9 planes of 8 blocks fit the SM -- and are read from the parameter
// planes in global memory (L1/L2-cached, coalesced) otherwise: with 6
// horizons they would take 54 KB per block and cap the SM at 4 blocks.
//
// HS_FR holds 1 - the step's runoff fractions, which the warp evaluates packed
// at the top of each step's soil moisture; with the parameters in global memory a plane of
// one pointer per thread (each thread's parameter planes) follows the horizon
// planes, so that a lane can read another lane's SMs and beta.
enum HorizonPlane : int { HS_SM = 0, HS_RSMS, HS_RDEN, HS_FR, HS_PAR0, HS_PLANES_ALL = HS_PAR0 + 5 };
__host__ __device__ constexpr bool hs_params_shared(int HL) { return HL <= 3; }
__host__ __device__ constexpr int hs_planes(int HL) { return hs_params_shared(HL) ? HS_PLANES_ALL : HS_PAR0; }
// dynamic shared memory of a block of B threads
__host__ __device__ constexpr size_t hs_bytes(int HL, int B)
{
    return (size_t)hs_planes(HL) * HL * B * sizeof(double) + (hs_params_shared(HL) ? 0 : (size_t)B * sizeof(void *));
}

// exp(beta * log(smh / SMs)) lies in [0, 1] for eps < smh <= SMs when SMs is
// finite and beta is finite and > 0 (integer tests on the bits)
__device__ __forceinline__ bool sm_frac_bounded(double sms, double beta)
{
    return hm_abs_bits(hm_d2b(sms)) < 0x7ff0000000000000ULL && hm_d2b(beta) - 1 < 0x7fefffffffffffffULL;
}

// position of the r-th (0-based) set bit of mask (r < popc(mask))
__device__ __forceinline__ int nth_set_bit(unsigned mask, int r)
{
    int pos = 0;
#pragma unroll
    for (int w = 16; w >= 1; w >>= 1) {
        const int c = __popc(mask & ((1u << w) - 1u));
        if (r >= c) {
            r -= c;
            mask >>= w;
            pos += w;
        }
    }
    return pos;
}


// LEAN: compiled for PET input (cases -1, 0) and the Feddes stress (soil-moisture
// cases 1, 4) only -- the configurations of the throughput workloads -- so that
// the Hargreaves / Priestley-Taylor / Penman-Monteith and Jarvis code is not in
// the instruction stream and the register allocation.
//
// cell_chain_item advances cell k of member m (both in range) of the launch
// described by `a`.  HL sizes the shared-memory horizon planes; DYN takes the
// horizon count from a.n_horizons (<= HL) at run time, so that one launch can
// serve contexts with different horizon counts (the fused multi-context
// launch); otherwise it is HL.
template <int HL, bool FLUX, bool LEAN, bool DYN>
__device__ __forceinline__ void cell_chain_item(const CellArgs &a, const int m, const int k)
{
    const int H = DYN ? a.n_horizons : HL;
    const int64_t N = a.n_cells;
    const StepInfo *steps = a.steps;
    bool reset_sm = a.reset_sm != 0;
    if (a.member_step0) {
        const int32_t b = a.member_step0[m];
        if (b < 0) { // idle member slot: no state update, zero runoff
            for (int t = 0; t < a.n_steps; ++t) a.tro[(size_t)t * a.n_members * N + (size_t)m * N + k] = 0.0;
            return;
        }
        if (!bc_ok(BC_STEP_ROW, (long long)b + a.step_shift + a.n_steps - 1, a.n_step_rows)) return;
        steps += b + a.step_shift;
        reset_sm = a.reset_ok && (b + a.step_shift == 0);
    }
    const int np = n_param_planes(H);
    const int ns = n_state_planes(H);
    const double *P = a.params + (size_t)m * np * N + k;
    double *S = a.states + (size_t)m * ns * N + k;
    auto par = [&](int plane) { return __ldg(P + (size_t)plane * N); };

    extern __shared__ double hsm[];
    const int tb = threadIdx.x, B = blockDim.x;
    auto hs = [&](int plane, int h) -> double & { return hsm[(plane * HL + h) * B + tb]; };
    // the per-horizon parameters, groups 0..4 = fRoots, SMs, FC, PW, beta
    auto hp = [&](int g, int h) -> double {
        if constexpr (hs_params_shared(HL)) return hs(HS_PAR0 + g, h);
        else return __ldg(P + (size_t)(P_HORIZON + g * H + h) * N);
    };
    const double **hptr = reinterpret_cast<const double **>(hsm + (size_t)hs_planes(HL) * HL * B);
    if constexpr (!hs_params_shared(HL)) hptr[tb] = P;
    const bool feddes = LEAN || (a.proc_sm == 1 || a.proc_sm == 4);
    CellRegs c;
    const double c2 = a.c2TSTu;
    c.fsealed = par(P_FSEALED);
    c.fnotsealed = 1.0 - c.fsealed;
    c.ddinc = par(P_DDINC);
    c.ddmax_s = par(P_DDMAX) * c2;   // mo_mhm.f90:463
    c.ddnopre_s = par(P_DDNOPRE) * c2; // mo_mhm.f90:464
    c.dd_thr = (c.ddmax_s - c.ddnopre_s) / c.ddinc; // mo_snow_accum_melt.f90:137
    c.tthresh = par(P_TTHRESH);
    c.sthresh = par(P_STHRESH);
    c.uthresh = par(P_UTHRESH);
    c.karst = par(P_KARST);
    c.alpha1 = 1.0 + par(P_ALPHA); // mo_runoff.f90:139
    c.k1s = c2 / par(P_K1);        // mo_mhm.f90:484
    c.kps = c2 / par(P_KP);
    c.k0s = c2 / par(P_K0);
    c.k2s = c2 / par(P_K2);        // mo_mhm.f90:488
    c.jarvis = par(P_JARVIS);
    c.fasp = par(P_FASP);
    c.harsam = par(P_HARSAM);
    c.lat_rad = (a.proc_pet == 1) ? kDeg2Rad * __ldg(a.latitude + k) : 0.0;
    c.r_sthresh = hm_recip_of(c.sthresh);
    c.r_jarvis = hm_recip_of(c.jarvis);
    bool frac_bounded = true; // every horizon's runoff fraction is in [0, 1]
#pragma unroll 1
    for (int h = 0; h < H; ++h) {
        if constexpr (hs_params_shared(HL)) {
            for (int g = 0; g < 5; ++g) hs(HS_PAR0 + g, h) = __ldg(P + (size_t)(P_HORIZON + g * H + h) * N);
        }
        const double sms = hp(1, h), fc = hp(2, h), pw = hp(3, h);
        hs(HS_RSMS, h) = hm_b2d(hm_recip_of(sms));
        hs(HS_RDEN, h) = hm_b2d(hm_recip_of(feddes ? fc - pw : sms - pw)); // mo_soil_moisture.f90:358, :435
        hs(HS_SM, h) = reset_sm ? 0.5 * fc : S[(size_t)(S_SM + h) * N];
        frac_bounded = frac_bounded && sm_frac_bounded(sms, hp(4, h));
    }
    c.interc = S[(size_t)S_INTERC * N];
    c.snow = S[(size_t)S_SNOW * N];
    c.seal = S[(size_t)S_SEAL * N];
    c.unsat = S[(size_t)S_UNSAT * N];
    c.sat = S[(size_t)S_SAT * N];

    const bool sealed = c.fsealed > 0.0;           // frac_sealed > 0 (parameter only)
    const bool sthresh_pos = c.sthresh > kEps;     // water_thresh_sealed > eps (parameter only)
    const bool dd_thr_ok = !hm_isnan_i(c.dd_thr);  // prec <= NaN is false
    int cur_key = -1;
    double imax = 0.0, petlai = 0.0, petsurf = 0.0, evap = 0.0;
    uint64_t r_imax = 0, r_evap = 0;
    int cur_doy = -1;
    double rad = 0.0;
    const size_t out_stride = (size_t)a.n_members * N;
    double *tro = a.tro + (size_t)m * N + k;
    // aggregated flux/state outputs (flux variant): running sums in device
    // memory, one [member][cell] plane per output variable
    const OutArgs &o = a.out;
    double *oacc = nullptr;
    int ocnt = 0, oslot = 0;
    int64_t ott_w = -1;
    if constexpr (FLUX) {
        if (o.n_planes > 0) {
            oacc = o.acc + (size_t)m * N + k;
            ocnt = o.cnt0;
            oslot = o.slot0;
            if (o.tt_w) ott_w = o.tt_w[m];
        }
    }
    // non-finite detection, integer operations only: a double is NaN or Inf
    // iff its sign-cleared bits are >= 0x7ff0...0, i.e. iff adding 2^52 to
    // them carries into bit 63; the OR over the steps keeps any such carry
    constexpr uint64_t kExpOne = 0x0010000000000000ull;
    uint64_t nonfin = 0;
    auto oadd = [&](int plane, double x) {
        double *q = oacc + (size_t)plane * out_stride;
        *q = *q + x; // OutputVariable%data = data + value, src/common/mo_nc_output.f90:140-149
    };

    for (int t = 0; t < a.n_steps; ++t) {
        const StepInfo si = steps[t];
        const int month = si.month;
        // the month (evap_coeff) and the LAI entry (iLAI: the month, or the
        // step's entry of a gridded LAI series) as one key: their parameters
        // are reloaded together when either changes
        const int key = ((int)si.lai << 4) | month;
        if (key != cur_key) {
            cur_key = key;
            evap = a.tab.evap[month - 1]; // evap_coeff of the calendar month
            r_evap = hm_recip_of(evap);
            if (!a.lai_series) { // iLAI = month: the monthly LAI slots
                imax = par(P_MAXINTER + month - 1);
                // petLAIcorFactor (proc_pet -1) or PrieTayAlpha (proc_pet 2) of the LAI month
                if (a.proc_pet == -1 || a.proc_pet >= 2) petlai = par(P_PETLAI + month - 1);
                if (!LEAN && a.proc_pet == 3) petsurf = par(P_PET2 + month - 1); // surfResist of the LAI month
            } else {             // a gridded LAI series: its entry iLAI
                if (!bc_ok(BC_LAI_STEP, si.lai - 1, a.n_lai)) break;
                const size_t NL = (size_t)a.n_lai * N;
                const double *ls = a.lai_series + (size_t)m * lai_groups(a.proc_pet) * NL + (size_t)(si.lai - 1) * N + k;
                imax = __ldg(ls);
                if (a.proc_pet == -1 || a.proc_pet >= 2) petlai = __ldg(ls + NL);
                if (!LEAN && a.proc_pet == 3) petsurf = __ldg(ls + 2 * NL);
            }
            r_imax = hm_recip_of(imax);
        }
        if (kBoundsChecked && !bc_ok(BC_FORCING_ROW, a.member_step0 ? a.step_shift + t : si.row - a.row_base,
                                     a.n_forc_rows))
            break;
        const size_t f = (size_t)(a.member_step0 ? a.step_shift + t : si.row - a.row_base) * N + k;
        // output weights: write_output runs after the calendar has advanced, so
        // it reads fSealed / soilMoistSat of the NEXT step's land-cover scene
        // (src/mHM/mo_mhm_interface_run.f90:621-629, 698-727)
        bool oon = false, ow = false;
        double ofs = 0.0, ofns = 0.0;
        if constexpr (FLUX) {
            const int64_t tt = o.tt_base + t;
            oon = oacc != nullptr && tt > o.warm_steps;
            ow = oon && tt == ott_w;
            ofs = ow ? o.w_fsealed[(size_t)m * N + k] : c.fsealed;
            ofns = 1.0 - ofs; // run_cfg%L1_fNotSealed = 1 - L1_fSealed (:239)
        }
        // ---- meteo for the step (mo_meteo_handler.f90:915-1285) ----
        double pv = 0.0;
        if (a.proc_pet == 0) {
            pv = c.fasp * __ldg(a.pet + f);
        } else if (a.proc_pet == -1) {
            pv = petlai * __ldg(a.pet + f);
        } else if constexpr (LEAN) {
        } else if (a.proc_pet == 2) { // Rn = max(L1_netrad, 0), src/meteo/mo_meteo_handler.f90:1080-1085
            const double rn = __ldg(a.netrad + f);
            pv = pet_priestly(petlai, rn > 0.0 ? rn : 0.0, __ldg(a.temp + f));
        } else if (a.proc_pet == 3) { // aeroResist / wind speed, eabs in kPa, :1087-1095
            const double rn = __ldg(a.netrad + f);
            pv = pet_penman(rn > 0.0 ? rn : 0.0, __ldg(a.temp + f), __ldg(a.eabs + f) / 1000.0,
                            petlai / __ldg(a.wind + f), petsurf);
        } else {
            if (si.doy != cur_doy) {
                cur_doy = si.doy;
                rad = extraterr_rad_approx(cur_doy, c.lat_rad);
            }
            pv = c.fasp * pet_hargreaves(c.harsam, __ldg(a.temp + f), __ldg(a.tmax + f), __ldg(a.tmin + f), rad);
        }
        double pet, temp, prec;
        if (a.is_hourly) {
            pet = pv;
            temp = __ldg(a.temp + f);
            prec = __ldg(a.pre + f);
        } else if (a.w_pet) {
            // temporal_disagg_meteo_weights (mo_meteo_temporal_tools.f90:32-50) with
            // L1_*_weights(k, month, hour + 1), mo_meteo_handler.f90:1102-1107, 1183-1189,
            // 1265-1270; temperature corrected by T0 = 273.15 K
            const size_t wi = ((size_t)si.hour * 12 + (size_t)(month - 1)) * N + k;
            pet = (pv + 0.0) * __ldg(a.w_pet + wi) - 0.0;
            temp = (__ldg(a.temp + f) + kT0) * __ldg(a.w_temp + wi) - kT0;
            prec = (__ldg(a.pre + f) + 0.0) * __ldg(a.w_pre + wi) - 0.0;
        } else { // temporal_disagg_*_daynight, mo_meteo_temporal_tools.f90:66-161
            const int mi = month - 1;
            const double nd = a.nTstepDay;
            if (nd > 1.0) {
                const bool isday = (si.dflags & SF_ISDAY) != 0;
                pet = 2.0 * pv * (isday ? a.tab.fday_pet[mi] : a.tab.fnight_pet[mi]) / nd;
                temp = __ldg(a.temp + f) + (isday ? a.tab.fday_temp[mi] : a.tab.fnight_temp[mi]);
                prec = 2.0 * __ldg(a.pre + f) * (isday ? a.tab.fday_prec[mi] : a.tab.fnight_prec[mi]) / nd;
            } else {
                pet = pv;
                temp = __ldg(a.temp + f);
                prec = __ldg(a.pre + f);
            }
        }

        // ---- canopy_interc, mo_canopy_interc.f90:75-133 ----
        // Branches that only pick between values are written as hm_sel (an
        // integer select of the bits): a double select or a merge of doubles
        // after a short if/else is issued on the FP64 pipe, the bottleneck.
        double throughfall, aet_can;
        {
            const double aux = c.interc + prec;
            const bool full = hm_ge(aux, imax);
            throughfall = hm_sel(full, aux - imax, 0.0);
            c.interc = hm_sel(full, imax, aux);
            aet_can = 0.0;
            if (hm_gt(imax, kEps)) aet_can = pet * hm_pow(hm_div_r(c.interc, imax, r_imax), kTwoThird);
            // a negative storage gives pow() = NaN: these two tests keep IEEE NaN semantics
            aet_can = hm_sel(hm_lt_ieee(aet_can, 0.0), 0.0, aet_can);
            const bool keep = hm_gt_ieee(c.interc, aet_can);
            const double rest = c.interc - aet_can;
            aet_can = hm_sel(keep, aet_can, c.interc);
            c.interc = hm_sel(keep, rest, 0.0);
        }
        // ---- snow_accum_melt, mo_snow_accum_melt.f90:70-158 ----
        double prec_effect, melt;
        {
            const bool warm = hm_gt(temp, c.tthresh);
            const double rain = hm_sel(warm, throughfall, 0.0);
            const double snowf = hm_sel(warm, 0.0, throughfall);
            melt = 0.0;
            if (warm) {
                double snow_left = 0.0;
                if (hm_gt0(c.snow)) { // the degree-day factor only matters here
                    const bool low = dd_thr_ok && hm_le(prec, c.dd_thr);
                    const double dd = hm_sel(low, c.ddnopre_s + c.ddinc * prec, c.ddmax_s);
                    const double aux = dd * (temp - c.tthresh);
                    const bool all = hm_gt(aux, c.snow);
                    melt = hm_sel(all, c.snow, aux);
                    snow_left = hm_sel(all, 0.0, c.snow - aux);
                }
                c.snow = snow_left;
            } else {
                c.snow = c.snow + snowf;
            }
            prec_effect = melt + rain;
        }
        // ---- the horizons' runoff fractions exp(beta log(SM / SMs)),
        // mo_soil_moisture.f90:230-234 ----
        // Each depends on its horizon's start-of-step soil moisture and on
        // parameters only, so the warp evaluates them ahead of the horizon
        // loop, packed: the (lane, horizon) pairs of the lanes that need them
        // are spread over all lanes of the warp, a pass of the warp per 32
        // pairs instead of one per horizon.  A lane whose effective
        // precipitation is +0 -- and whose fractions are known to lie in
        // [0, 1] -- needs none: every horizon's input is then +0, and
        // pin * (1 - frac) is +0 for every such fraction, so the loop takes
        // frac = 0.
        // The same function of the same operands gives the same bits on any
        // lane.
        const bool need_frac = hm_d2b(prec_effect) != 0 || !frac_bounded;
        {
            const unsigned gm = __activemask();
            __syncwarp(gm); // the soil moisture the lanes wrote last step is visible
            const unsigned nm = __ballot_sync(gm, need_frac);
            unsigned lt;
            asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
            const int G = __popc(gm), n_tasks = __popc(nm) * H, wb = tb & ~31;
#pragma unroll 1
            for (int t = __popc(gm & lt); t < n_tasks; t += G) {
                const int r = t / H, h = t - r * H;
                const int ol = wb + nth_set_bit(nm, r); // the lane the pair belongs to
                const double smh = hsm[(HS_SM * HL + h) * B + ol];
                double sms, beta;
                if constexpr (hs_params_shared(HL)) {
                    sms = hsm[((HS_PAR0 + 1) * HL + h) * B + ol];
                    beta = hsm[((HS_PAR0 + 4) * HL + h) * B + ol];
                } else {
                    const double *Po = hptr[ol];
                    sms = __ldg(Po + (size_t)(P_HORIZON + H + h) * N);
                    beta = __ldg(Po + (size_t)(P_HORIZON + 4 * H + h) * N);
                }
                double fr = 0.0;
                if (hm_gt(smh, kEps) && !hm_gt(smh, sms))
                    fr = hm_exp(beta * hm_log(hm_div_r(smh, sms, hm_d2b(hsm[(HS_RSMS * HL + h) * B + ol]))));
                hsm[(HS_FR * HL + h) * B + ol] = 1.0 - fr;
            }
            __syncwarp(gm); // the fractions are visible to their lanes
        }
        // ---- soil_moisture, mo_soil_moisture.f90:176-286 ----
        double runoff_sealed = 0.0;
        double infil_last;
        double aet_sealed_act = 0.0, aet_soil = 0.0; // for the optional flux outputs
        {
            if (sealed) {
                const double tmp = c.seal + prec_effect;
                const bool over = hm_gt(tmp, c.sthresh);
                runoff_sealed = hm_sel(over, tmp - c.sthresh, 0.0);
                c.seal = hm_sel(over, c.sthresh, tmp);
                double aet_sealed = DBL_MAX;
                if (sthresh_pos) {
                    aet_sealed = (hm_div_r(pet, evap, r_evap) - aet_can) * hm_div_r(c.seal, c.sthresh, c.r_sthresh);
                    aet_sealed = hm_sel(hm_lt0(aet_sealed), 0.0, aet_sealed);
                }
                const bool keep = hm_gt(c.seal, aet_sealed);
                const double rest = c.seal - aet_sealed;
                if constexpr (FLUX) aet_sealed_act = hm_sel(keep, aet_sealed, c.seal);
                c.seal = hm_sel(keep, rest, 0.0);
            }
            double infil = prec_effect; // prec_effec_soil of horizon 1
            double aet_above = 0.0;     // masked running sum of positive aet above
            const double demand = pet - aet_can;
#pragma unroll 1
            for (int h = 0; h < H; ++h) {
                const double pin = infil;
                const double sms = hp(1, h);
                double smh = hs(HS_SM, h);
                if (!hm_gt(smh, sms)) { // else the horizon passes its input on: infil stays pin
                    // 1 - frac_runoff, evaluated above (frac_runoff = 0 when smh <= eps),
                    // or 1 - 0 for a lane that needs none
                    const double tmp = pin * hm_sel(need_frac, hs(HS_FR, h), 1.0);
                    const double filled = smh + tmp;
                    const bool over = hm_gt(filled, sms);
                    // pin + (smh - sms) or pin - tmp, as one addition: pin - tmp is
                    // pin + (-tmp) exactly, so the select picks the second operand
                    infil = pin + hm_sel(over, smh - sms, hm_neg(tmp));
                    smh = hm_sel(over, sms, filled);
                }
                // demand minus the positive aet above (x - (+0) == x: no test for h == 0)
                double aet = demand - aet_above;
                const double froots = hp(0, h), pw = hp(3, h), fc = hp(2, h);
                double stress;
                if (feddes) {
                    const bool wet = hm_ge(smh, fc);
                    stress = hm_sel(wet, froots, 0.0);
                    // mo_soil_moisture.f90:358
                    if (!wet && hm_gt(smh, pw))
                        stress = hm_div_r(froots * (smh - pw), fc - pw, hm_d2b(hs(HS_RDEN, h)));
                } else {
                    // with SMs == PW the quotient can be NaN (0 / 0): IEEE
                    // comparisons then leave the stress at 0 as the oracle does
                    double th = hm_div_r(smh - pw, sms - pw, hm_d2b(hs(HS_RDEN, h)));
                    th = hm_sel(hm_lt_ieee(th, 0.0), 0.0, th);
                    th = hm_sel(hm_gt_ieee(th, 1.0), 1.0, th);
                    const bool wet = hm_ge_ieee(th, c.jarvis);
                    stress = hm_sel(wet, froots, 0.0);
                    if (!wet && hm_lt_ieee(th, c.jarvis)) stress = froots * hm_div_r(th, c.jarvis, c.r_jarvis);
                }
                aet = aet * stress;
                aet = hm_sel(hm_lt0(aet), 0.0, aet);
                // enough: storage smh - aet, aet kept; else aet = smh - eps and
                // storage eps -- one subtraction serves both cases
                const bool enough = hm_gt(smh, aet);
                const double d = smh - hm_sel(enough, aet, kEps);
                aet = hm_sel(enough, aet, d);
                smh = hm_sel(enough, d, kEps);
                smh = hm_sel(hm_lt(smh, kEps), kEps, smh);
                hs(HS_SM, h) = smh;
                aet_above = hm_sel(hm_gt0(aet), aet_above + aet, aet_above);
                if constexpr (FLUX) {
                    aet_soil = aet_soil + aet;
                    if (oon) { // soil_infil_L<h>, aET_L<h> (mo_write_fluxes_states.f90:414-426)
                        if (o.plane[OF_INFIL] >= 0) oadd(o.plane[OF_INFIL] + h, infil * ofns);
                        if (o.plane[OF_AET_L] >= 0) oadd(o.plane[OF_AET_L] + h, aet * ofns);
                    }
                }
            }
            infil_last = infil;
        }
        // ---- runoff_unsat_zone, mo_runoff.f90:74-154 ----
        double fast = 0.0, slow = 0.0, base, perc;
        {
            c.unsat = c.unsat + infil_last;
            if (hm_gt(c.unsat, c.uthresh)) fast = hm_min_sel(c.k0s * (c.unsat - c.uthresh), c.unsat - kEps);
            c.unsat = c.unsat - fast; // - (+0) keeps the value when nothing flows
            if (hm_gt(c.unsat, kEps)) slow = hm_min_sel(c.k1s * hm_pow(c.unsat, c.alpha1), c.unsat - kEps);
            c.unsat = c.unsat - slow;
            perc = c.kps * c.unsat;
            // if the store cannot supply kp * unsat, perc = unsat: both branches of
            // the reference add perc * karstLoss to the saturated store
            const bool rest = hm_gt(c.unsat, perc);
            perc = hm_sel(rest, perc, c.unsat);
            c.sat = c.sat + perc * c.karst;
            c.unsat = hm_sel(rest, c.unsat - perc, 0.0);
            if constexpr (FLUX) {
                if (a.flux_aet) {
                    const size_t fo = (size_t)t * out_stride + (size_t)m * N + k;
                    a.flux_aet[fo] = aet_can + c.fsealed * aet_sealed_act + c.fnotsealed * aet_soil;
                    a.flux_loss[fo] = c.fnotsealed * (perc - perc * c.karst);
                }
            }
        }
        // ---- runoff_sat_zone, mo_runoff.f90:191-212 ----
        {
            const bool pos = hm_gt0(c.sat);
            const double b0 = c.k2s * c.sat;
            base = hm_sel(pos, b0, 0.0);
            c.sat = hm_sel(pos, c.sat - b0, 0.0);
        }
        // ---- L1_total_runoff, mo_runoff.f90:248-274 ----
        const double q_total = ((base + slow + fast) * c.fnotsealed) + (runoff_sealed * c.fsealed);
        tro[(size_t)t * out_stride] = q_total;
        nonfin |= hm_abs_bits(hm_d2b(q_total)) + kExpOne;
        if constexpr (FLUX) {
            // mHM_updateDataset, src/mHM/mo_write_fluxes_states.f90:283-438
            if (oon) {
                const int8_t *pl = o.plane;
                if (pl[OF_INTERC] >= 0) oadd(pl[OF_INTERC], c.interc);
                if (pl[OF_SNOW] >= 0) oadd(pl[OF_SNOW], c.snow);
                if (pl[OF_SWC] >= 0)
                    for (int h = 0; h < H; ++h) oadd(pl[OF_SWC] + h, hs(HS_SM, h));
                if (pl[OF_SM] >= 0 || pl[OF_SM_ALL] >= 0) {
                    double ssm = 0.0, ssat = 0.0;
                    for (int h = 0; h < H; ++h) {
                        const double sat_h = ow ? o.w_sms[((size_t)m * H + h) * N + k] : hp(1, h);
                        if (pl[OF_SM] >= 0) oadd(pl[OF_SM] + h, hs(HS_SM, h) / sat_h);
                        ssm = ssm + hs(HS_SM, h);
                        ssat = ssat + sat_h;
                    }
                    if (pl[OF_SM_ALL] >= 0) oadd(pl[OF_SM_ALL], ssm / ssat);
                }
                if (pl[OF_SEAL] >= 0) oadd(pl[OF_SEAL], c.seal);
                if (pl[OF_UNSAT] >= 0) oadd(pl[OF_UNSAT], c.unsat);
                if (pl[OF_SAT] >= 0) oadd(pl[OF_SAT], c.sat);
                if (pl[OF_PET] >= 0) oadd(pl[OF_PET], pet);
                if (pl[OF_AET] >= 0) oadd(pl[OF_AET], aet_soil * ofns + aet_can + aet_sealed_act * ofs);
                if (pl[OF_Q] >= 0) oadd(pl[OF_Q], q_total);
                if (pl[OF_QD] >= 0) oadd(pl[OF_QD], runoff_sealed * ofs);
                if (pl[OF_QIF] >= 0) oadd(pl[OF_QIF], fast * ofns);
                if (pl[OF_QIS] >= 0) oadd(pl[OF_QIS], slow * ofns);
                if (pl[OF_QB] >= 0) oadd(pl[OF_QB], base * ofns);
                if (pl[OF_RECHARGE] >= 0) oadd(pl[OF_RECHARGE], perc * ofns);
                if (pl[OF_PRE_EFFECT] >= 0) oadd(pl[OF_PRE_EFFECT], prec_effect);
                if (pl[OF_QSM] >= 0) oadd(pl[OF_QSM], melt);
                ++ocnt; // OutputVariable%counter
                const int64_t tt = o.tt_base + t;
                if (out_writeout(o.interval, tt - o.warm_steps, tt, o.n_tt, si.dflags)) {
                    // writeVariableTimestep, src/common/mo_nc_output.f90:158-175
                    double *dst = o.out + (size_t)oslot * o.n_planes * out_stride + (size_t)m * N + k;
                    for (int v = 0; v < o.n_planes; ++v) {
                        double *q = oacc + (size_t)v * out_stride;
                        const double x = *q;
                        if (oslot < o.max_slots)
                            dst[(size_t)v * out_stride] = ((o.avg_mask >> v) & 1) ? x / (double)ocnt : x;
                        *q = 0.0;
                    }
                    ++oslot;
                    ocnt = 0;
                }
            }
        }
    }

    S[(size_t)S_INTERC * N] = c.interc;
    S[(size_t)S_SNOW * N] = c.snow;
    S[(size_t)S_SEAL * N] = c.seal;
    S[(size_t)S_UNSAT * N] = c.unsat;
    S[(size_t)S_SAT * N] = c.sat;
    auto chk = [&](double x) { nonfin |= hm_abs_bits(hm_d2b(x)) + kExpOne; };
    chk(c.interc);
    chk(c.snow);
    chk(c.seal);
    chk(c.unsat);
    chk(c.sat);
#pragma unroll 1
    for (int h = 0; h < H; ++h) {
        const double smh = hs(HS_SM, h);
        S[(size_t)(S_SM + h) * N] = smh;
        chk(smh);
    }
    if (a.nonfinite && (nonfin >> 63)) atomicOr(a.nonfinite + m, 1);
}

// Work items of a launch, by block: one member's 128 consecutive cells, or --
// when the members come in groups of 4 -- 32 consecutive cells of 4 members
// (one member per warp, so a warp still walks 32 neighbouring cells of one
// parameter set).  The blocks of one cell tile are consecutive in launch order
// and start together, so the forcing rows every member reads come from L1/L2
// after the first member group instead of from DRAM once per member.
__host__ __device__ constexpr bool member_tiles(int64_t n_members) { return n_members > 1 && n_members % 4 == 0; }

template <int H, int MINB, bool FLUX, bool LEAN>
__global__ void __launch_bounds__(128, MINB) cell_chain_kernel(const CellArgs a)
{
    const int64_t N = a.n_cells;
    int m, k;
    if (member_tiles(a.n_members)) {
        const int64_t n_groups = a.n_members / 4;
        const int64_t tile = blockIdx.x / n_groups;
        m = (int)(blockIdx.x - tile * n_groups) * 4 + (int)(threadIdx.x >> 5);
        const int64_t kk = tile * 32 + (threadIdx.x & 31);
        if (kk >= N) return;
        k = (int)kk;
    } else {
        const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
        if (gid >= N * a.n_members) return;
        m = (int)(gid / N);
        k = (int)(gid - (int64_t)m * N);
    }
    cell_chain_item<H, FLUX, LEAN, false>(a, m, k);
}

// The cell chain of several contexts in one persistent launch: a work queue
// of tiles (128 consecutive work items of one context), taken in queue order
// by the resident blocks with one atomic increment per tile.  Each block
// copies the tile's context description into shared memory and runs the same
// per-item code as cell_chain_kernel, so every item's arithmetic -- and
// result -- is that of the context's own launch.  No block waits on another:
// a block returns when the queue is empty.
template <int HL, bool LEAN, int MINB>
__global__ void __launch_bounds__(128, MINB) cell_chain_fused_kernel(const FusedCellArgs f)
{
    __shared__ CellArgs sa;
    __shared__ int32_t tile;
    for (;;) {
        if (threadIdx.x == 0) tile = atomicAdd(f.queue, 1);
        __syncthreads();
        const int32_t t = tile;
        if (t >= f.n_tiles) return;
        const uint32_t *src = reinterpret_cast<const uint32_t *>(f.args + __ldg(f.tile_ctx + t));
        uint32_t *dst = reinterpret_cast<uint32_t *>(&sa);
        for (int w = threadIdx.x; w < (int)(sizeof(CellArgs) / 4); w += blockDim.x) dst[w] = __ldg(src + w);
        __syncthreads();
        const int64_t gid = __ldg(f.tile_item0 + t) + threadIdx.x;
        const int64_t N = sa.n_cells;
        if (gid < N * sa.n_members) {
            const int m = (int)(gid / N);
            cell_chain_item<HL, false, LEAN, true>(sa, m, (int)(gid - (int64_t)m * N));
        }
        __syncthreads(); // the next tile may overwrite sa and the horizon planes
    }
}

// Launch with H as a template parameter (shared-memory size, loop bounds);
// MINB = resident blocks per SM the register allocation is sized for.
template <int MINB, bool FLUX, bool LEAN>
cudaError_t launch_cell_chain_h(const CellArgs &a, int H, cudaStream_t s)
{
    const int64_t n = (int64_t)a.n_cells * a.n_members;
    const int block = 128;
    const unsigned grid = member_tiles(a.n_members)
                              ? (unsigned)(((int64_t)a.n_cells + 31) / 32 * (a.n_members / 4))
                              : (unsigned)((n + block - 1) / block);
    const size_t smem = hs_bytes(H, block);
    switch (H) {
#define MHM_CASE(HH)                                                                                               \
    case HH:                                                                                                       \
        if (smem > 48 * 1024)                                                                                      \
            cudaFuncSetAttribute(cell_chain_kernel<HH, MINB, FLUX, LEAN>,                                          \
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);                          \
        cell_chain_kernel<HH, MINB, FLUX, LEAN><<<grid, block, smem, s>>>(a);                                      \
        break;
        MHM_CASE(1) MHM_CASE(2) MHM_CASE(3) MHM_CASE(4) MHM_CASE(5) MHM_CASE(6) MHM_CASE(7) MHM_CASE(8)
#undef MHM_CASE
    default:
        return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int MINB, bool FLUX = false>
cudaError_t launch_cell_chain_variant(const CellArgs &a, int H, cudaStream_t s)
{
    if constexpr (!FLUX) {
        const bool lean = (a.proc_pet == 0 || a.proc_pet == -1) && (a.proc_sm == 1 || a.proc_sm == 4);
        if (lean) return launch_cell_chain_h<MINB, false, true>(a, H, s);
    }
    return launch_cell_chain_h<MINB, FLUX, false>(a, H, s);
}

} // namespace
} // namespace mhm
