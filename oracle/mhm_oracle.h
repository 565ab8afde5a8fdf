/*
 * mhm_oracle.h -- CPU restatement of the mHM / mRM hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the GPU
 * implementation in mhm_gb300/: only tests/, __graft_entry__.smoke() and the
 * CPU-baseline leg of bench.py may load it.  Nothing in the product links or
 * calls it.
 *
 * Each function restates one reference routine (cited at its definition in
 * mhm_oracle.c), keeping the reference's evaluation order, branch conditions,
 * eps_dp = epsilon(1d0) and Fortran real**real semantics.  The reference is
 * compiled by gfortran without FMA contraction, so this file is compiled with
 * -ffp-contract=off.  Two builds exist:
 *   liboracle_hmath.so -- exp/log/pow from mhm_gb300/csrc/hmath.h (the same
 *                         elementary functions the GPU uses: bitwise parity);
 *   liboracle_libm.so  -- exp/log/pow from the C library (glibc), i.e. the
 *                         functions gfortran calls: the reference-semantics
 *                         build, compared at 1e-9 relative.
 * Arrays: 0-based C pointers; index values stored in them (L1_L11_Id,
 * netPerm, fromN, toN, gauge nodes) are 1-based as in Fortran.  2-D arrays
 * (cells, horizons) are column-major as in the reference: element (k, h) is at
 * [h * nCells + k].
 */
#ifndef MHM_ORACLE_H
#define MHM_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- process routines (scalar, as in the reference) ---- */
void ora_canopy_interc(double pet, double interc_max, double precip, double *interc,
                       double *throughfall, double *evap_canopy);
void ora_snow_accum_melt(double deg_day_incr, double deg_day_max, double deg_day_noprec,
                         double prec, double temperature, double temperature_thresh,
                         double thrfall, double *snow_pack, double *deg_day, double *melt,
                         double *prec_effect, double *rain, double *snow);
double ora_feddes_et_reduction(double sm, double fc, double pw, double froots);
double ora_jarvis_et_reduction(double sm, double sat, double pw, double froots, double c1);
void ora_soil_moisture(int processCase, int nH, double frac_sealed, double water_thresh_sealed,
                       double pet, double evap_coeff, const double *sm_sat, const double *frac_roots,
                       const double *sm_fc, const double *wilting_point, const double *sm_exponen,
                       double jarvis_thresh_c1, double aet_canopy, double prec_effec,
                       double *runoff_sealed, double *storage_sealed, double *infiltration,
                       double *soil_moist, double *aet, double *aet_sealed);
void ora_runoff_unsat_zone(double k1, double kp, double k0, double alpha, double karst_loss,
                           double pefec_soil, double unsat_thresh, double *sat_storage,
                           double *unsat_storage, double *slow_interflow, double *fast_interflow,
                           double *perc);
void ora_runoff_sat_zone(double k2, double *sat_storage, double *baseflow);
double ora_L1_total_runoff(double fsealed, double fast, double slow, double base, double direct);

double ora_extraterr_rad_approx(int doy, double latitude_rad);
double ora_pet_hargreaves(double HarSamCoeff, double HarSamConst, double tavg, double tmax,
                          double tmin, double latitude_deg, int doy);
double ora_sat_vap_pressure(double tavg);
double ora_slope_satpressure(double tavg);
double ora_pet_priestly(double alpha, double rn, double tavg);
double ora_pet_penman(double net_rad, double tavg, double act_vap_pressure, double aerodyn_resistance,
                      double bulksurface_resistance, double a_s, double a_sh);

double ora_disagg_meteo_weights(double day_val, double weight, double correction);
double ora_disagg_flux_daynight(int isday, double ntimesteps_day, double day_val, double fday,
                                double fnight);
double ora_disagg_state_daynight(int isday, double ntimesteps_day, double day_val, double fday,
                                 double fnight, int add_correction);

/* ---- calendar (mo_julian restated) ---- */
int32_t ora_julday(int32_t dd, int32_t mm, int32_t yy);
void ora_caldat(int32_t julian, int32_t *dd, int32_t *mm, int32_t *yy);
void ora_dec2date(double julian, int32_t *dd, int32_t *mm, int32_t *yy, int32_t *hh,
                  int32_t *nn, int32_t *ss);
/* Per-step calendar of a run, emulating datetimeinfo (init/increment) and the
 * dec2date(newTime - 0.5) calls of do_time_step.  For steps tt = 1..nSteps:
 * month[tt-1], hour, doy, day, year. */
void ora_step_calendar(int32_t jul_start, int32_t timestep, int32_t nSteps, int32_t *month,
                       int32_t *hour, int32_t *doy, int32_t *day, int32_t *year);
void ora_step_lai(int32_t jul_start, int32_t timestep, int32_t lai_mode, int32_t nSteps, int32_t *lai);
void ora_step_calendar_ex(int32_t jul_start, int32_t timestep, int32_t nSteps, int32_t *month,
                          int32_t *hour, int32_t *doy, int32_t *day, int32_t *year, int32_t *new_flags);

/* ---- routing ---- */
void ora_reg_rout(const double *param5, const double *length, const double *slope,
                  const double *fFPimp, int nLinks, double TS, double *C1, double *C2);
void ora_L11_runoff_acc(int nCells, int nNodes, const double *qAll, const double *efecArea,
                        const int32_t *L1_L11_Id, const double *L11_areaCell,
                        const int32_t *L11_L1_Id, int TS, int map_flag, double *qAcc);
/* qTIN, qTR: column-major (nNodes, 2), column IT1=0 holds the previous step. */
void ora_L11_routing(int nNodes, int nLinks, const int32_t *netPerm, const int32_t *fromN,
                     const int32_t *toN, const double *C1, const double *C2, const double *qOUT,
                     double *qTIN, double *qTR, double *Qmod);
/* src/mRM/mo_mrm_pre_routing.f90:179-214 */
void ora_add_inflow(int nInflowGauges, const int32_t *InflowHeadwater, const int32_t *InflowNodeList,
                    const double *QInflow, double *qOut);
/* L11_routing with inflow gauges (src/mRM/mo_mrm_routing.f90:380-481) */
void ora_L11_routing_ex(int nNodes, int nLinks, const int32_t *netPerm, const int32_t *fromN, const int32_t *toN,
                        const double *C1, const double *C2, const double *qOUT, int nInflowGauges,
                        const int32_t *InflowHeadwater, const int32_t *InflowNodeList, double *qTIN, double *qTR,
                        double *Qmod);
/* L11_set_network_topology: links from the L11 D8 directions (mRM codes). fDir11 and
 * the returned ids use the L11 grid packed column-major over the mask (cells 1..nCells),
 * cellCoor[k] = (row, col) 1-based.  Returns nLinks; fromN/toN sized nCells. */
int ora_L11_set_network_topology(int nrows, int ncols, const int32_t *id2d /*[ncols][nrows]*/,
                                 int nCells, const int32_t *cellRow, const int32_t *cellCol,
                                 const int32_t *fDir11, int32_t *fromN, int32_t *toN);
/* L11_routing_order, literal O(nLinks^2) sweep.  Outputs sized nNodes:
 * netPerm (1-based link ids in routing order), rOrder (rank of each link). */
void ora_L11_routing_order(int nNodes, int nOutlets, const int32_t *fromN, const int32_t *toN,
                           int32_t *netPerm, int32_t *rOrder);
int ora_L11_routing_order_listed(int nNodes, int nOutlets, const int32_t *fromN, const int32_t *toN,
                                 int32_t *netPerm, int32_t *rOrder);

/* Routing case 2 (mrm_update_param, src/mRM/mo_mrm_mpr.f90:241-329): K = length /
 * celerity per link, the routing time step TSrout [s] = given_TS(locate(given_TS,
 * min K)), C1/C2 with xi = 0.  Returns TSrout. */
double ora_update_param_case2(double celerity, const double *length, int nLinks, double *C1, double *C2);
double ora_update_param_links(const double *link_celerity, double celerity, const double *length, int nLinks,
                              double *C1, double *C2);
double ora_link_celerity(double slope_factor, const double *path_slope, int n);

/* ---- whole-domain run (the mhm_eval time loop for one domain) ---- */
typedef struct {
    int32_t nCells, nH, nNodes, nOutlets, timestep;
    int32_t proc_sm;      /* processMatrix(3,1): 1..4 */
    int32_t proc_pet;     /* processMatrix(5,1): -1, 0, 1, 2 */
    int32_t proc_rout;    /* processMatrix(8,1): 0, 1, 2 or 3 */
    int32_t nTstepForcingDay; /* 24 (hourly) or 1 (daily) */
    int32_t read_states;  /* 1: states (and C1/C2) come from a restart */
    int32_t jul_start;    /* simPer%julStart */
    int32_t map_flag;     /* routing resolution >= hydrology resolution */
    int32_t nGauges;
    int32_t pad_;
    const double *evap_coeff;                 /* [12] */
    const double *fday_prec, *fnight_prec;    /* [12] */
    const double *fday_pet, *fnight_pet;      /* [12] */
    const double *fday_temp, *fnight_temp;    /* [12] */
    const double *l1_area_km2;                /* [nCells] CellArea * 1e-6 */
    const int32_t *l1_l11_id;                 /* [nCells] */
    const double *l11_area_km2;               /* [nNodes] */
    const int32_t *l11_l1_id;                 /* [nNodes] */
    const int32_t *net_perm, *from_n, *to_n;  /* [nNodes] (valid 1..nLinks) */
    const double *length, *slope, *ffp_imp;   /* [nLinks] */
    const double *rout_param;                 /* [5] (case 1) or [1] celerity [m s-1] (case 2) */
    const int32_t *gauge_node;                /* [nGauges] */
    const double *latitude;                   /* [nCells] degrees */
    const double *link_celerity;              /* [nLinks] L11_celerity (routing case 3) */
    /* read_meteo_weights: hourly weights L1_{pre,pet,temp}_weights(cell, month, hour),
     * [24][12][nCells]; NULL: day/night ratios */
    const double *pre_w, *pet_w, *temp_w;
    /* inflow gauges (mRM InflowGauge): L11 node (1-based) and headwater flag of
     * each, and their daily discharge [m3 s-1], inflow_q[(day - inflow_day0) * nInflow + g]
     * for days inflow_day0 .. inflow_day0 + inflow_ndays - 1 (day = iDischargeTS) */
    int32_t nInflow, inflow_day0, inflow_ndays, pad2_;
    const int32_t *inflow_node, *inflow_headwater;
    const double *inflow_q;
    /* timeStep_LAI_input: 0 (or 1) monthly LAI slots indexed by the calendar
     * month; -1 / -2 / -3 a gridded LAI series, its index raised at every new
     * day / month / year of the run (the first step counts as new).  n_lai:
     * the series' length (the LAI-indexed parameters then hold n_lai entries
     * per cell). */
    int32_t lai_mode, n_lai;
} ora_domain;

typedef struct {
    const double *fSealed, *alpha, *degDayInc, *degDayMax, *degDayNoPre, *fAsp, *HarSamCoeff;
    const double *karstLoss, *kFastFlow, *kSlowFlow, *kBaseFlow, *kPerco;
    const double *jarvis_c1, *tempThresh, *unsatThresh, *sealedThresh;
    const double *maxInter;        /* [12][nCells] (column-major (nCells, 12)) */
    const double *petLAIcorFactor; /* [12][nCells] or NULL */
    const double *fRoots, *SMs, *FC, *PW, *beta; /* [nH][nCells] */
    const double *PrieTayAlpha;    /* [12][nCells] Priestley-Taylor alpha (proc_pet 2) or NULL */
    const double *aeroResist, *surfResist; /* [12][nCells] Penman-Monteith resistances (proc_pet 3) or NULL */
} ora_params;

typedef struct {
    double *interc, *snowpack, *sealSTW, *SM /*[nH][nCells]*/, *unsat, *sat;
    double *qTIN, *qTR;   /* [2][nNodes] column-major (nNodes, 2) */
    double *qOUT, *Qmod;  /* [nNodes] */
    double *C1, *C2;      /* [nNodes] (links 1..nLinks used) */
    double *run_to_rout;  /* [nCells] routing case 2 with a routing step of several
                             model steps: runoff summed since the last routing (or NULL) */
} ora_state;

/* Forcing rows: row r of pre/temp/pet/tmin/tmax is [r][nCells]; the row used at
 * step tt is iMeteoTS(tt) - forc_row0 (iMeteoTS as in update_timestep, 1-based). */
typedef struct {
    const double *pre, *temp, *pet, *tmin, *tmax;
    int32_t forc_row0;
    int32_t n_rows;
    const double *netrad; /* net radiation [W m-2] (proc_pet 2, 3) or NULL */
    const double *eabs, *windspeed; /* absolute vapour pressure [Pa], wind speed [m s-1] (proc_pet 3) */
} ora_forcing;

/* Aggregated outputs of the run (mhm_interface_run_write_output,
 * src/mHM/mo_mhm_interface_run.f90:641-742): mHM's outputFlxState variables
 * (src/mHM/mo_write_fluxes_states.f90) and mRM's Qrouted
 * (src/mRM/mo_mrm_write_fluxes_states.f90), summed per step after the
 * warm-up and written at the end of each interval (src/common/mo_nc_output.f90:
 * 140-175, src/common/mo_common_datetime_type.f90:157-185).  Counters and sums
 * carry over between ora_run_ex calls. */
typedef struct {
    int32_t interval, interval_mrm;  /* timeStep_model_outputs, timeStep_model_outputs_mrm */
    int32_t warm_steps, n_time_steps;
    int32_t flags[21];               /* outputFlxState(1..21) (18, neutrons, not supported) */
    int32_t qrouted;                 /* outputFlxState_mrm(1) */
    int32_t max_slots;
    int32_t n_planes;                /* set by ora_output_planes */
    int32_t plane[22];               /* first plane of variable f (1-based), -1 if off */
    int32_t counter, counter_mrm, n_slots, n_slots_mrm;
    int32_t tt_w;                    /* step whose outputs use w_fsealed / w_sms (0: none) */
    int32_t pad_;
    double *acc, *out;               /* [n_planes][nCells], [max_slots][n_planes][nCells] */
    int32_t *slot_tt;                /* [max_slots] step that closed each interval */
    double *acc_mrm, *out_mrm;       /* [nNodes], [max_slots][nNodes] */
    int32_t *slot_tt_mrm;
    const double *w_fsealed, *w_sms; /* [nCells], [nH][nCells] */
} ora_output;

/* Plane layout in the order of the output file's variables; returns n_planes
 * (or -1 for an unsupported variable). */
int ora_output_planes(ora_output *o, int nH);

/* Run steps tt = tt0 .. tt0+nT-1 (1-based, tt0 >= 1).  Outputs (any may be NULL):
 * q_gauge[nT][nGauges], total_runoff[nT][nCells], qmod[nT][nNodes].
 * nthreads <= 0: OpenMP default.  Returns 0 on success. */
int ora_run(const ora_domain *d, const ora_params *p, ora_state *s, const ora_forcing *f,
            int32_t tt0, int32_t nT, double *q_gauge, double *total_runoff, double *qmod,
            int nthreads);
/* ora_run plus aggregated outputs (out may be NULL); returns -5 when an
 * interval would overflow max_slots */
int ora_run_ex(const ora_domain *d, const ora_params *p, ora_state *s, const ora_forcing *f,
               int32_t tt0, int32_t nT, double *q_gauge, double *total_runoff, double *qmod,
               int nthreads, ora_output *out);

/* Set the reference's default initial states (mo_init_states.f90:258-345,
 * mo_mrm_init.f90:453-499).  horizon_depth[nH] in mm. */
void ora_default_states(const ora_domain *d, const double *horizon_depth, ora_state *s);

/* which elementary-function build this is: 0 = hmath, 1 = libm */
int ora_math_kind(void);

/* ---- multiscale parameter regionalisation (mhm_oracle_mpr.c) ---- */
/* One land-cover scene, iFlag_soilDB = 0.  L0 cells are packed column-major
 * over mask0 (0-based k0); id0_2d[col * nrows0 + row] is k0 or -1 outside the
 * mask.  L1 cell k1 covers L0 rows up1..down1 and columns left1..right1
 * (1-based, inclusive) and holds nsub1 valid L0 cells. */
typedef struct {
    int32_t nCells0, nrows0, ncols0, nCells1;
    int32_t nH;        /* nSoilHorizons_mHM (>= 2) */
    int32_t nSoil;     /* soil types in the database (ids 1..nSoil) */
    int32_t maxHor;    /* stride of the per-soil horizon arrays */
    int32_t nGeo;      /* geological units */
    int32_t proc_sm;   /* processMatrix(3,1): 1..4 */
    int32_t proc_pet;  /* processMatrix(5,1): -1, 0, 1, 2 */
    int32_t n_soil_params; /* processMatrix(3,2): 17, 18, 22 or 21 */
    int32_t nLAI;      /* entries of LAI0 (size(LAI0, 2)); 0 means 12 */
    double fracSealed_cityArea;
    const int32_t *id0_2d;                        /* [ncols0 * nrows0] */
    const int32_t *up1, *down1, *left1, *right1, *nsub1; /* [nCells1] */
    const int32_t *LCover0, *soilId0, *geoUnit0;  /* [nCells0], 1-based class ids */
    const double *slope_emp0, *Asp0, *y0;         /* [nCells0] */
    const double *LAI0;                           /* [nLAI][nCells0] */
    const int32_t *present, *nHor, *nTill;        /* [nSoil] */
    const double *sand, *clay, *DbM;              /* [nSoil][maxHor] */
    const double *RZdepth;                        /* [nSoil] */
    const double *Wd;                             /* [nSoil][nH][maxHor] */
    const double *horizonDepth;                   /* [nH], as left by ora_soil_weights */
    const int32_t *geoUnitList, *geoUnitKar;      /* [nGeo] */
} ora_mpr_domain;

/* global parameters by process, in namelist order */
typedef struct {
    const double *interc;    /* [1] canopyInterceptionFactor */
    const double *snow;      /* [8] */
    const double *soil;      /* [n_soil_params] */
    const double *runoff;    /* [1] imperviousStorageCapacity */
    const double *pet;       /* [3] aspect, [4] Hargreaves-Samani, [5] LAI correction */
    const double *interflow; /* [5] */
    const double *perc;      /* [3] */
    const double *geo;       /* [nGeo] */
} ora_gamma;

/* L1 outputs: per-cell [nCells1], per-horizon [nH][nCells1], monthly [12][nCells1] */
typedef struct {
    double *fSealed, *alpha, *degDayInc, *degDayMax, *degDayNoPre, *fAsp, *HarSamCoeff;
    double *karstLoss, *kFastFlow, *kSlowFlow, *kBaseFlow, *kPerco;
    double *jarvis_c1, *tempThresh, *unsatThresh, *sealedThresh;
    double *maxInter, *petLAIcorFactor;
    double *fRoots, *SMs, *FC, *PW, *beta;
    double *PrieTayAlpha; /* [12][nCells1] (proc_pet 2) or NULL */
    double *aeroResist, *surfResist; /* [12][nCells1] (proc_pet 3) or NULL */
} ora_mpr_out;

int ora_mpr(const ora_mpr_domain *d, const ora_gamma *g, ora_mpr_out *o);
void ora_hydro_cond(const double *param4, double sand, double clay, double *Ks);
void ora_genuchten(const double *param6, double sand, double clay, double Db, double *thetaS,
                   double *n, double *alpha);
void ora_field_cap(double Ks, double thetaS, double n, double *thetaFC);
void ora_pwp(double n, double alpha, double thetaS, double *thetaPWP);
/* Wd [nSoil][nH][maxHor]; horizonDepth[nH-1] is overwritten (see the source) */
int ora_soil_weights(int nSoil, int maxHor, const int32_t *nHor, const double *UD, const double *LD,
                     const double *RZdepth, int nH, double *horizonDepth, double *Wd);
int ora_slope_emp(int n, const double *slope, double *slope_emp);

#ifdef __cplusplus
}
#endif
#endif
