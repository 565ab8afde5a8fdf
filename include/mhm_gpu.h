/*
 * mhm_gpu.h -- C ABI of the GB300 implementation of mHM's per-cell water
 * balance and mRM's Muskingum routing (libmhm_gpu.so).
 *
 * The reference has no C interface: its hot path is a set of Fortran module
 * procedures.  Each entry point below replaces one of them, with the same
 * argument meaning, and is what an iso_c_binding interface module on the
 * Fortran side binds.
 *
 * Conventions
 *   - Every function returns an int status: MHM_OK (0) or a negative MHM_ERR_*
 *     code; mhm_last_error() gives a message.  Arguments are validated on the
 *     host before anything is launched.
 *   - Arrays follow the reference's layout: L1 cells are packed column-major
 *     over the mask (src/common/mo_grid.f90:145-150), 2-D (cell, horizon) and
 *     (cell, month) arrays are column-major, i.e. element (k, h) is at
 *     [h * n_cells + k]; index VALUES (L1_L11_Id, netPerm, fromN, toN, gauge
 *     nodes) are 1-based as in Fortran.
 *   - Host pointers are borrowed for the duration of the call only, except
 *     the forcing set by mhm_set_forcing, which is read by the following
 *     mhm_run calls.
 *   - A context is used by one host thread at a time (the reference is not
 *     reentrant either); separate contexts may run concurrently.
 *   - A context owns all its device memory.  Several parameter sets
 *     ("members", e.g. a calibration ensemble) can share one domain and one
 *     forcing: member m has its own effective parameters, states and outputs.
 *   - All state arithmetic is IEEE FP64.
 */
#ifndef MHM_GPU_H
#define MHM_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MHM_OK 0
#define MHM_ERR_INVALID (-1)     /* bad argument or shape */
#define MHM_ERR_CUDA (-2)        /* CUDA runtime error or no device */
#define MHM_ERR_OOM (-3)         /* device allocation failed */
#define MHM_ERR_TIMEOUT (-4)     /* a bounded device wait ran out */
#define MHM_ERR_NAN (-5)         /* non-finite state or forcing detected */
#define MHM_ERR_UNSUPPORTED (-6) /* process option not implemented */
#define MHM_ERR_BOUNDS (-7)      /* bounds-checked build: an index taken from data was out of range */

/* forcing kinds for mhm_set_forcing (the reference's L1_pre, L1_temp, L1_pet,
 * L1_tmin, L1_tmax of src/meteo/mo_meteo_handler.f90) */
#define MHM_FORC_PRE 0
#define MHM_FORC_TEMP 1
#define MHM_FORC_PET 2
#define MHM_FORC_TMIN 3
#define MHM_FORC_TMAX 4
#define MHM_FORC_NETRAD 5    /* L1_netrad [W m-2] (proc_pet = 2, 3)                   */
#define MHM_FORC_EABS 6      /* L1_absvappress [Pa], Penman-Monteith PET (proc_pet = 3) */
#define MHM_FORC_WINDSPEED 7 /* L1_windspeed [m s-1] (proc_pet = 3)                   */

typedef struct mhm_ctx mhm_ctx;

/* One basin: what mHM's initialisation (mhm_interface_init, mrm_init) hands
 * to the time loop.  Replaces the module globals read by do_time_step
 * (src/mHM/mo_mhm_interface_run.f90:341-638) and mRM_routing
 * (src/mRM/mo_mrm_routing.f90:104-110). */
typedef struct {
    int32_t n_cells;             /* level1%nCells                              */
    int32_t n_horizons;          /* nSoilHorizons_mHM (1..8)                   */
    int32_t n_nodes;             /* level11%nCells                             */
    int32_t n_outlets;           /* L11_nOutlets                               */
    int32_t timestep;            /* model time step [h] (mhm.nml timestep)     */
    int32_t proc_soilmoist;      /* processMatrix(3,1): 1..4                   */
    int32_t proc_pet;            /* processMatrix(5,1): -1, 0, 1, 2 or 3       */
    int32_t proc_routing;        /* processMatrix(8,1): 0, 1 (Muskingum), 2
                                    (Muskingum with a routing time step chosen
                                    from a constant celerity) or 3 (from each
                                    link's celerity)                           */
    int32_t n_tstep_forcing_day; /* 24 (hourly forcing) or 1 (daily forcing)   */
    int32_t jul_start;           /* simPer%julStart (Julian day number)        */
    int32_t map_flag;            /* routing resolution >= hydrology resolution */
    int32_t n_gauges;            /* domain_mrm%nGauges                         */
    int32_t n_members;           /* parameter sets run together (>= 1)         */
    int32_t read_states;         /* 1: states come from a restart (no SM reset
                                    at tt == 1, C1/C2 not regenerated)         */
    const double *evap_coeff;    /* [12] mhm.nml &panEvapo                      */
    const double *fday_prec, *fnight_prec; /* [12] &nightDayRatio             */
    const double *fday_pet, *fnight_pet;   /* [12]                            */
    const double *fday_temp, *fnight_temp; /* [12]                            */
    const double *l1_area_km2;   /* [n_cells] level1%CellArea * 1e-6           */
    const int32_t *l1_l11_id;    /* [n_cells] L1_L11_Id                        */
    const double *l11_area_km2;  /* [n_nodes] level11%CellArea * 1e-6          */
    const int32_t *l11_l1_id;    /* [n_nodes] L11_L1_Id (used if !map_flag)    */
    const int32_t *net_perm;     /* [n_nodes] L11_netPerm (1..nLinks valid)    */
    const int32_t *from_n;       /* [n_nodes] L11_fromN                        */
    const int32_t *to_n;         /* [n_nodes] L11_toN                          */
    const double *length;        /* [nLinks] L11_length [m]                    */
    const double *slope;         /* [nLinks] L11_slope                         */
    const double *ffp_imp;       /* [nLinks] L11_nLinkFracFPimp                */
    const int32_t *gauge_node;   /* [n_gauges] gaugeNodeList                   */
    const double *latitude;      /* [n_cells] level1%y (only for proc_pet = 1) */
} mhm_domain_desc;

/* L1 effective parameters of one member: the L1_* arrays of
 * src/MPR/mo_mpr_global_variables.f90 that mHM() reads
 * (src/mHM/mo_mhm_interface_run.f90:405-451), for one land-cover scene. */
typedef struct {
    const double *fSealed, *alpha, *degDayInc, *degDayMax, *degDayNoPre;
    const double *fAsp, *HarSamCoeff;
    const double *karstLoss, *kFastFlow, *kSlowFlow, *kBaseFlow, *kPerco;
    const double *jarvis_thresh_c1, *tempThresh, *unsatThresh, *sealedThresh;
    const double *maxInter;        /* [12 * n_cells] (cell, LAI month)          */
    const double *petLAIcorFactor; /* [12 * n_cells] or NULL (proc_pet = -1)    */
    const double *fRoots, *soilMoistSat, *soilMoistFC, *wiltingPoint, *soilMoistExp; /* [H * n_cells] */
    const double *PrieTayAlpha;    /* [12 * n_cells] or NULL (proc_pet = 2, L1_PrieTayAlpha); it shares
                                      the device planes of petLAIcorFactor, which is then not read back */
    const double *aeroResist, *surfResist; /* [12 * n_cells] or NULL (proc_pet = 3, L1_aeroResist of
                                              the scene and L1_surfResist); aeroResist shares those planes too */
} mhm_eff_params;

/* Restart state of one member: the fields of src/mHM/mo_restart.f90:146-258
 * (L1_Inter, L1_snowPack, L1_sealSTW, L1_soilMoist, L1_unsatSTW, L1_satSTW)
 * and src/mRM/mo_mrm_restart.f90:231-272 (L11_qOUT, L11_qTIN, L11_qTR,
 * L11_Qmod, L11_C1, L11_C2), packed as in the reference's memory. */
typedef struct {
    double *interc, *snowpack, *sealSTW, *unsatSTW, *satSTW; /* [n_cells]        */
    double *soilMoist;                                       /* [H * n_cells]    */
    double *qOUT, *Qmod;                                     /* [n_nodes]        */
    double *qTIN, *qTR;            /* [2 * n_nodes]: column 1 = previous step     */
    double *C1, *C2;                                         /* [n_nodes]        */
} mhm_restart;

/* Context lifetime.  Replaces mhm_interface_init's domain set-up
 * (src/mHM/mo_mhm_interface.F90:37-228): validates the network (netPerm must
 * be a topological order of the links) and builds the device-side routing
 * levels.  Selects device `device` (-1: current). */
int mhm_ctx_create(const mhm_domain_desc *desc, int32_t device, mhm_ctx **out);
int mhm_ctx_destroy(mhm_ctx *ctx);
const char *mhm_last_error(const mhm_ctx *ctx);
/* cudaStream_t of the context (work of all calls is ordered on it). */
void *mhm_ctx_stream(mhm_ctx *ctx);

/* Effective parameters of `member` (the restart path of
 * mhm_interface_run_prepare, src/mHM/mo_mhm_interface_run.f90:221-231). */
int mhm_set_eff_params(mhm_ctx *ctx, int32_t member, const mhm_eff_params *p);
/* The member's effective parameters copied back into the (host) arrays the
 * struct points to; NULL fields are skipped.  For checking mhm_mpr against
 * the reference's L1_* arrays. */
int mhm_get_eff_params(mhm_ctx *ctx, int32_t member, const mhm_eff_params *p);

/* Gridded LAI series (timeStep_LAI_input, src/common/mo_common_datetime_type.f90:
 * 138-155): mode 0 (or 1) keeps the 12 monthly LAI slots of the effective
 * parameters (iLAI = month); -1 / -2 / -3 read the LAI-indexed parameters --
 * maxInter, the petLAIcorFactor / PrieTayAlpha / aeroResist group and
 * surfResist -- from a series of n_lai entries, iLAI counting the days /
 * months / years from the run's first step (tt = 1 is entry 1).  The series
 * starts zeroed; mhm_set_lai_params fills a member's entries, each array
 * [n_lai][n_cells] or NULL (zeros).  Only the groups the context's PET case
 * reads are stored (maxInter always; the second group for PET -1, 2, 3; the
 * third for 3): the others are ignored and read back as zeros.  A run whose
 * last step lies beyond the series fails with MHM_ERR_INVALID. */
int mhm_set_lai_series(mhm_ctx *ctx, int32_t mode, int32_t n_lai);
int mhm_set_lai_params(mhm_ctx *ctx, int32_t member, const double *max_inter, const double *pet_lai,
                       const double *surf_resist);
/* The member's series entries read back (each pointer may be NULL); mhm_mpr
 * with gridded L0 LAI of the series' length writes them (the reference's
 * L1_maxInter, L1_petLAIcorFactor / L1_PrieTayAlpha / L1_aeroResist and
 * L1_surfResist over size(LAI0, 2) entries, src/MPR/mo_multi_param_reg.f90:
 * 1142, 1266-1281). */
int mhm_get_lai_params(mhm_ctx *ctx, int32_t member, double *max_inter, double *pet_lai, double *surf_resist);

/* Floodplain impervious fraction of the links [nLinks] for the land-cover
 * scene that starts (L11_nLinkFracFPimp(:, iLC) of src/mRM/mo_mrm_routing.f90
 * follows the scene of the current year); the next mhm_set_routing_params /
 * mhm_mpr computes C1/C2 with it. */
int mhm_set_link_fpimp(mhm_ctx *ctx, const double *ffp_imp);

/* read_meteo_weights = .true.: daily forcing is spread over the day with
 * hourly weights instead of the day/night ratios (temporal_disagg_meteo_weights,
 * src/meteo/mo_meteo_temporal_tools.f90:32-50, called from
 * src/meteo/mo_meteo_handler.f90:1102-1107, 1183-1189, 1265-1270):
 * x = (x_day + c) * w(cell, month, hour) - c with c = 273.15 K for the
 * temperature and 0 otherwise.  Each array is L1_{pre,pet,temp}_weights
 * (cell, month, hour) in the reference's column-major order, i.e.
 * [24][12][n_cells]; the three together, or all NULL to return to the
 * day/night ratios.  Hourly forcing ignores them, as the reference does. */
int mhm_set_meteo_weights(mhm_ctx *ctx, const double *pre_w, const double *pet_w, const double *temp_w);

/* Muskingum coefficients C1/C2 of `member` from the five routing parameters
 * (reg_rout, src/mRM/mo_mrm_mpr.f90:61-119; evaluated on the device).  With
 * routing case 2 rout_param5[0] is the streamflow celerity [m s-1]
 * (mrm_update_param, src/mRM/mo_mrm_mpr.f90:241-329): the routing time step is
 * the largest of the reference's allowed steps not above the shortest link's
 * travel time; shorter than the model step, each step's runoff is routed
 * that many times and the step's discharge is their mean; longer, runoff is
 * summed over that many model steps, routed once and the result stands for
 * each of them (then every mhm_run must cover whole routing steps). */
int mhm_set_routing_params(mhm_ctx *ctx, int32_t member, const double *rout_param5);
/* Routing case 3 (mrm_update_param, src/mRM/mo_mrm_mpr.f90:241-329): the
 * celerity of each link [n_links] (m s-1) for `member`, as L11_calc_celerity
 * derives it from the L0 river path of the link and the slope_factor
 * parameter (src/mRM/mo_mrm_net_startup.f90:2212-2423; see
 * mhm_gb300.routing.link_celerity).  K = length / celerity per link; the
 * routing step and C1/C2 then follow as in case 2.  (mhm_mpr leaves case-3
 * coefficients to this call.) */
int mhm_set_link_celerity(mhm_ctx *ctx, int32_t member, const double *celerity);

/* Inflow gauges (InflowGauge of mRM's configuration; add_inflow,
 * src/mRM/mo_mrm_pre_routing.f90:179-214, called from mRM_routing at
 * src/mRM/mo_mrm_routing.f90:234-241, and the headwater cut inside
 * L11_routing, :447-452).  n gauges at the L11 nodes node[n] (1-based):
 * headwater[g] != 0 adds the gauge's discharge to the node's own runoff
 * (InflowGaugeHeadwater = .true.); otherwise the discharge replaces that
 * runoff and every link draining into the node passes no water on.  Gauges
 * act in list order.  n = 0 removes them.  At most 64 gauges. */
int mhm_set_inflow_gauges(mhm_ctx *ctx, int32_t n, const int32_t *node, const int32_t *headwater);
/* Daily discharge [m3 s-1] of the inflow gauges, q[(d - day0) * n + g] for
 * days d = day0 .. day0 + n_days - 1, where model step tt belongs to day
 * ceiling(tt / (24 / timestep)) (iDischargeTS, InflowGauge%Q(iDischargeTS, :),
 * src/mHM/mo_mhm_interface_run.f90:463-511).  Copied to the device; a run
 * must lie inside the days given. */
int mhm_set_inflow_discharge(mhm_ctx *ctx, int32_t day0, int32_t n_days, const double *q);

/* Default initial states (fluxes_states_default_init,
 * src/mHM/mo_init_states.f90:258-345, and fluxes_states_default_init_routing,
 * src/mRM/mo_mrm_init.f90:453-499).  horizon_depth[n_horizons] in mm. */
int mhm_init_states(mhm_ctx *ctx, int32_t member, const double *horizon_depth);

/* Forcing rows row0 .. row0+n_rows-1 (1-based forcing step index iMeteoTS of
 * src/meteo/mo_meteo_handler.f90:575-620), layout [n_rows][n_cells].
 * on_device = 0: host memory, copied to the device inside mhm_run (pinned
 * memory from mhm_host_alloc overlaps the copies with compute);
 * on_device = 1: device memory that stays valid until the next
 * mhm_set_forcing of that kind. */
int mhm_set_forcing(mhm_ctx *ctx, int32_t kind, int32_t row0, int32_t n_rows, const double *data,
                    int32_t on_device);

/* Advance all members by time steps tt0 .. tt0+n_steps-1 (1-based as the
 * reference's tt): n_steps x do_time_step (src/mHM/mo_mhm_interface_run.f90:
 * 341-638) without file output, i.e. meteo for the step, the mHM() cell chain
 * (src/mHM/mo_mhm.f90:229-521) and mRM_routing (src/mRM/mo_mrm_routing.f90:
 * 104-303).  q_gauge (host, may be NULL): gauge discharge [m3 s-1],
 * laid out [member][gauge][step] (per member the column-major
 * mRM_runoff(step, gauge) of the reference).  Blocks until done. */
int mhm_run(mhm_ctx *ctx, int32_t tt0, int32_t n_steps, double *q_gauge);

/* Asynchronous variant: enqueue the steps and return; the routing of one call
 * overlaps the cell chain of the next.  q_gauge and host forcing must stay
 * valid until mhm_sync returns; state access and the set-up calls
 * synchronise first.  Per-step outputs (mhm_enable_outputs) need mhm_run. */
int mhm_run_async(mhm_ctx *ctx, int32_t tt0, int32_t n_steps, double *q_gauge);
/* Wait for all enqueued work of the context. */
int mhm_sync(mhm_ctx *ctx);
/* Without waiting: *done = 1 if all work enqueued so far has completed on
 * the device (mhm_sync then returns at once and finishes the host side:
 * gauge series into the caller's buffers), else 0.  For a serving loop that
 * advances several contexts independently.  No counterpart in the
 * reference. */
int mhm_poll(mhm_ctx *ctx, int32_t *done);

/* Members at different model steps (continuous batching of independent runs
 * of one basin): member m advances its own steps member_tt0[m] ..
 * member_tt0[m]+n_steps-1 (calendar and SM initialisation at its step 1 as in
 * mhm_run), all members reading rows 0..n_steps-1 of the device forcing
 * window set by mhm_set_forcing; member_tt0[m] <= 0 leaves member m idle (its
 * cell and routing states untouched, its discharge zero).  Hourly steps with hourly forcing
 * only.  Each member's results equal a run of that member alone from the
 * same states over the same forcing rows.  Enqueues and returns like
 * mhm_run_async. */
int mhm_run_members_async(mhm_ctx *ctx, const int32_t *member_tt0, int32_t n_steps, double *q_gauge);

/* Autotuner (no counterpart in the reference): times n_steps from step tt0
 * with every combination of the cell-chain register variant (sized for 4, 6
 * or 8 resident blocks per SM) and the routing wavefront sub-chunk (4, 8 or
 * 16 steps), restoring all members' states before each trial and after the
 * last, and keeps the fastest for the context's later runs.  Needs the
 * forcing for those steps.  ms_out (may be NULL) receives the 9 trial times
 * in (variant, sub-chunk) order. */
int mhm_autotune(mhm_ctx *ctx, int32_t tt0, int32_t n_steps, int32_t *occ_out, int32_t *sub_out, double *ms_out);

/* How a context launches its work (no counterpart in the reference). */
typedef struct mhm_launch_config {
    int32_t cell_blocks_per_sm; /* cell-chain register variant: 4, 6 or 8 resident blocks per SM */
    int32_t route_sub_steps;    /* steps per routing wavefront sub-chunk, 1..16 */
    int32_t chunk_steps;        /* most time steps per chunk (0: the device-memory budget decides) */
    int32_t route_cluster;      /* routing of a chunk: 0 = one launch per wavefront tick (replayed
                                   from a CUDA graph); 4, 8 or 16 = all ticks in one launch, each
                                   thread-block cluster of that many CTAs walking the wavefront of
                                   its members with a hardware cluster barrier between ticks */
} mhm_launch_config;
int mhm_set_launch_config(mhm_ctx *ctx, const mhm_launch_config *cfg);
int mhm_get_launch_config(mhm_ctx *ctx, mhm_launch_config *cfg);
/* mhm_autotune over one more knob, the time-chunk length: each of the
 * n_chunk_choices chunk lengths (0 = as the memory budget allows; at most 8)
 * is tried with every register variant and routing sub-chunk.  A run is
 * split into chunks whose routing overlaps the next chunk's cell chain, so
 * shorter chunks trade launches for overlap.  n_chunk_choices = 0 keeps the
 * context's chunk length.  ms_out (may be NULL) receives 9 trial times per
 * chunk length, in (chunk length, variant, sub-chunk) order; best_out the
 * configuration kept. */
int mhm_autotune_ex(mhm_ctx *ctx, int32_t tt0, int32_t n_steps, int32_t n_chunk_choices,
                    const int32_t *chunk_choices, mhm_launch_config *best_out, double *ms_out);
/* The routing launch mode by timing n_steps from tt0 with the context's
 * other settings (states restored afterwards): route_cluster 0, 4, 8 and 16
 * in that order (ms_out, may be NULL: 4 trial times); the fastest is kept and
 * written to *cluster_out (may be NULL).  Contexts without routing keep 0. */
int mhm_autotune_route(mhm_ctx *ctx, int32_t tt0, int32_t n_steps, int32_t *cluster_out, double *ms_out);

/* Device-resident restart states: n_slots snapshot slots per context (each
 * one member's cell and routing states); save/load copy on the device,
 * ordered after the context's enqueued work (warm starts without a host
 * round trip). */
/* Failure status of each member since the last call: status[m] = MHM_OK, or
 * MHM_ERR_NAN when a state or the total runoff of member m became NaN or
 * infinite in any step (checked by the cell chain on the integer pipe at no
 * measurable cost).  Waits for the enqueued work, then clears the flags.
 * Returns MHM_ERR_NAN if any member failed (message names them), else
 * MHM_OK.  The reference has no such check -- a non-finite value silently
 * propagates there (its only error path is error_message -> stop,
 * src/MPR/mo_multi_param_reg.f90:314,422); here one bad member of a batch
 * or one bad request of a serving loop can be failed on its own while the
 * others continue. */
int mhm_member_status(mhm_ctx *ctx, int32_t *status);

/* Bounds-checked build (the library built with -DMHM_BOUNDS_CHECK, loaded as
 * libmhm_gpu_bc.so): every index a kernel takes from data -- forcing rows,
 * the member step table, network tables, L1 <-> L11 mappings, gauge and
 * inflow positions, inflow days, soil keys, LAI classes and geology units of
 * the L0 codes -- is tested before the access; a failed test records (site,
 * index) in a device status word (the first one wins) and skips the access,
 * never trapping.  The status words belong to the device: the next
 * mhm_sync or mhm_device_status on that device reports MHM_ERR_BOUNDS.
 * mhm_bounds_checked() is 1 in that build, 0 otherwise.  mhm_device_status
 * waits for the context's work and returns MHM_OK or MHM_ERR_BOUNDS with
 * the site (1 forcing row, 2 member step row, 3 L1 cell of a node, 4 L1 cell
 * of an L11 cell, 5 upstream position, 6 qOUT row, 7 gauge position,
 * 8 inflow gauge position, 9 inflow day, 10 soil key, 11 LAI class,
 * 12 geology unit, 13 gridded-LAI entry, 99 self-test) and index; both may be NULL.
 * mhm_bounds_selftest runs one failing test with no access behind it (site
 * 99, index 7) so a caller can check the reporting path; MHM_ERR_UNSUPPORTED
 * in other builds.  (No reference counterpart: the reference's debug builds
 * use the Fortran compilers' run-time checks, src/CMakeLists.txt:71.) */
int mhm_bounds_checked(void);
int mhm_device_status(mhm_ctx *ctx, int32_t *site, int64_t *index);
int mhm_bounds_selftest(mhm_ctx *ctx);

/* Batches of contexts (no counterpart in the reference, whose farm of
 * parameter sets and domains runs them one after another or on separate MPI
 * ranks, src/common/mo_common_MPI_tools.F90:39-69): one call enqueues a
 * chunk of per-member steps on each of n contexts -- each exactly as
 * mhm_run_members_async(ctxs[i], member_tt0[i], n_steps, q_gauge[i]) -- with
 * the cell chain of all of them in ONE persistent launch on the batch's
 * stream: the resident blocks take 128-item tiles of all contexts from a
 * device work queue (tiles of contexts with more soil horizons first), so
 * basins of very different sizes fill the GPU together; accumulation and
 * routing then run on each context's own streams.  Every context must live
 * on the batch's device, use device forcing, take the call in one chunk and
 * have no per-step or aggregated outputs enabled; all must share the process
 * cases' code path (PET input with the Feddes stress, or not).  Results are
 * bit-identical to the contexts' own launches.  Poll or synchronise each
 * context as after mhm_run_members_async; q_gauge may be NULL or hold NULLs. */
typedef struct mhm_batch mhm_batch;
int mhm_batch_create(int32_t device, mhm_batch **out);
int mhm_batch_destroy(mhm_batch *b);
const char *mhm_batch_last_error(const mhm_batch *b);
int mhm_batch_run_members(mhm_batch *b, int32_t n, mhm_ctx *const *ctxs, const int32_t *const *member_tt0,
                          int32_t n_steps, double *const *q_gauge);

int mhm_snapshot_alloc(mhm_ctx *ctx, int32_t n_slots);
int mhm_snapshot_save(mhm_ctx *ctx, int32_t member, int32_t slot);
int mhm_snapshot_load(mhm_ctx *ctx, int32_t slot, int32_t member);

/* Per-step L1 total runoff [mm TS-1] and L11 discharge of the last mhm_run:
 * optional outputs enabled before the run (adds HBM traffic). */
int mhm_enable_outputs(mhm_ctx *ctx, int32_t total_runoff, int32_t qmod);
/* total_runoff [n_steps][member][n_cells]; qmod [member][n_steps][n_nodes] */
int mhm_get_outputs(mhm_ctx *ctx, double *total_runoff, double *qmod);

/* Per-step cell fluxes of the following mhm_run calls (the aET and
 * percolation outputs of src/mHM/mo_write_fluxes_states.f90, per step instead
 * of aggregated): total actual evapotranspiration (canopy + sealed share +
 * soil share, mm per step) and the karstic percolation loss
 * (1 - fSealed) * perc * (1 - karstLoss), both [n_steps][member][n_cells].
 * With precipitation and total runoff they close the cell water balance. */
int mhm_enable_fluxes(mhm_ctx *ctx, int32_t on);
int mhm_get_fluxes(mhm_ctx *ctx, double *aet, double *loss);

/* Aggregated per-cell flux/state outputs, the mHM_Fluxes_States file's
 * variables (replaces mHM_OutputDataset / mHM_updateDataset / writeTimestep,
 * src/mHM/mo_write_fluxes_states.f90:48-438 and src/common/mo_nc_output.f90:
 * 140-262, driven from mhm_interface_run_write_output,
 * src/mHM/mo_mhm_interface_run.f90:641-742).
 *
 * flags[i] = outputFlxState(i+1) of mhm_outputs.nml: 1 interception,
 * 2 snowpack, 3 SWC_L<h>, 4 SM_L<h>, 5 SM_Lall, 6 sealedSTW, 7 unsatSTW,
 * 8 satSTW, 9 PET, 10 aET, 11 Q, 12 QD, 13 QIf, 14 QIs, 15 QB, 16 recharge,
 * 17 soil_infil_L<h>, 18 neutrons (refused: process 10 is not built),
 * 19 aET_L<h>, 20 preEffect, 21 Qsm.  Per-horizon variables give one plane
 * per horizon.  Planes follow the file's variable order (1, 2, 3, 4, 5, 6, 7,
 * 8, 9, 10, ..., 17, 19, 20, 21).  States (1-8) are written as the mean over
 * the interval, fluxes as its sum, in mm (per step) like the reference.
 *
 * Steps tt <= warming_steps add nothing; step tt closes an interval when
 * timestep_model_outputs > 0 divides tt - warming_steps, when the next step
 * starts a new day / month / year (-1 / -2 / -3), and always at
 * tt == n_time_steps (0: only then).  The device keeps up to max_slots
 * closed intervals, [slot][plane][member][n_cells]; a run that would close
 * more than the free slots is refused: read them first.  Enabling again (or
 * with cfg == NULL, off) clears sums and slots.  Runs with per-member steps
 * (mhm_run_members_async) refuse aggregated outputs. */
typedef struct {
    int32_t timestep_model_outputs; /* > 0: every n steps; 0: at the end; -1 daily; -2 monthly; -3 yearly */
    int32_t max_slots;              /* closed intervals held on the device between reads */
    int64_t warming_steps;          /* warmingDays * steps per day */
    int64_t n_time_steps;           /* steps of the simulation period */
    int32_t flags[21];              /* outputFlxState(1..21); Qrouted: flags[0] (flags[1] river temperature refused) */
    int32_t pad_;
} mhm_output_config;
int mhm_enable_flux_state_outputs(mhm_ctx *ctx, const mhm_output_config *cfg);
/* Copies the closed intervals ([n_slots][n_planes][member][n_cells]) and the
 * model step that closed each, then frees the slots.  out == NULL: only
 * *n_slots (and *n_planes) are set. */
int mhm_read_flux_state_outputs(mhm_ctx *ctx, double *out, int64_t *slot_tt, int32_t max_slots, int32_t *n_slots,
                                int32_t *n_planes);
/* mRM's Qrouted output: the L11 discharge of every node, mean over each
 * interval (mRM_OutputDataset / mRM_updateDataset,
 * src/mRM/mo_mrm_write_fluxes_states.f90:48-140), same interval rules with
 * timeStep_model_outputs_mrm; out is [n_slots][member][n_nodes] in L11 node
 * order.  Needs routing. */
int mhm_enable_routed_outputs(mhm_ctx *ctx, const mhm_output_config *cfg);
int mhm_read_routed_outputs(mhm_ctx *ctx, double *out, int64_t *slot_tt, int32_t max_slots, int32_t *n_slots);
/* The reference writes a step's outputs after advancing its calendar, so the
 * last step before a land-cover scene change is weighted with the NEXT
 * scene's fSealed (QD, QIf, QIs, QB, recharge, aET, soil_infil, aET_L) and
 * soilMoistSat (SM_L, SM_Lall) (src/mHM/mo_mhm_interface_run.f90:621-629,
 * 698-727).  Outputs of model step tt of `member` use these values
 * (fsealed [n_cells], soil_moist_sat [n_horizons][n_cells]) instead of the
 * member's current parameters; tt < 1 clears the override. */
int mhm_set_output_weights(mhm_ctx *ctx, int32_t member, int64_t tt, const double *fsealed,
                           const double *soil_moist_sat);

/* Restart state of one member (host buffers). */
int mhm_get_state(mhm_ctx *ctx, int32_t member, const mhm_restart *st);
int mhm_set_state(mhm_ctx *ctx, int32_t member, const mhm_restart *st);

/* One state or flux variable by the reference's pybind name
 * (pybind/src/wrapper.f90:569-777): "L1_INTER", "L1_SNOWPACK", "L1_SEALSTW",
 * "L1_SOILMOIST", "L1_UNSATSTW", "L1_SATSTW", "L11_QMOD", "L11_QOUT". */
int mhm_get_var(mhm_ctx *ctx, int32_t member, const char *name, double *out);

/* Per-kernel device time of the calls since the last reset, measured with
 * CUDA events on the context's stream.  kind: 0 cell chain, 1 L1->L11
 * accumulation, 2 routing, 3 everything between the first and last launch of
 * an mhm_run.  Timing is off unless enabled (it adds event records). */
int mhm_set_timing(mhm_ctx *ctx, int32_t on);
int mhm_get_timing(mhm_ctx *ctx, int32_t kind, int64_t *launches, double *total_ms);

/* L11 links from the L11 flow directions (host computation, no device
 * needed): replaces L11_set_network_topology
 * (src/mRM/mo_mrm_net_startup.f90:630-727).  Cell k (1-based, packed
 * column-major over the L11 mask) at grid row cell_row[k-1], column
 * cell_col[k-1] (1-based) drains into the cell its D8 code fdir[k-1]
 * (1, 2, 4, ..., 128 as moveDownOneCell steps them) points at; a cell that
 * points at itself (code 0, the outlet) gives no link.  id2d [ncols * nrows]
 * is the 1-based cell id of every grid cell, row index fastest (Fortran's
 * iD11(row, col)).  from_n / to_n [n_cells] receive L11_fromN / L11_toN in
 * cell order (-9999 past the last link), *n_links their number.
 * MHM_ERR_INVALID if a direction leaves the grid or the mask. */
int mhm_network_topology(int32_t nrows, int32_t ncols, const int32_t *id2d, int32_t n_cells, const int32_t *cell_row,
                         const int32_t *cell_col, const int32_t *fdir, int32_t *from_n, int32_t *to_n,
                         int32_t *n_links);

/* mRM's network start-up from level-0 flow data (host code, once per basin;
 * src/mRM/mo_mrm_net_startup.f90): the L11 grid over the L0 mask
 * (init_lowres_level, src/common/mo_grid.f90:58-183), L11_flow_direction
 * (:227-629, L11 coarser than L0), L11_set_network_topology (:630-727),
 * L11_routing_order (:728-886), L11_link_location (:887-1087),
 * L11_stream_features (:1233-1509: link length and slope >= 1e-4 along the
 * L0 river, the floodplain within deltaH = 5 m) and
 * L11_fraction_sealed_floodplain (:1510-1594), for cartesian grids
 * (iFlag_cordinate_sys = 0).  L0 grids use mHM's (x, y) order: nrows0 cells
 * west to east, ncols0 north to south, mask0[(j-1)*nrows0 + (i-1)], data
 * packed over the mask in that order; flow directions are mRM's codes
 * (1 E, 2 SE, 4 S, 8 SW, 16 W, 32 NW, 64 N, 128 NE as moveDownOneCell moves
 * on that grid).  lcover0 is [n_lc_scenes][n_cells0]; lc_class_imp the
 * sealed class (2). */
typedef struct mhm_l0_flow {
    int32_t nrows0, ncols0, factor, n_cells0;
    const uint8_t *mask0;
    const int32_t *fdir0, *facc0;
    const double *elev0;
    double cellsize0;
    int32_t n_lc_scenes, lc_class_imp;
    const int32_t *lcover0;
} mhm_l0_flow;
/* Outputs, allocated by the caller: n_nodes from mhm_l11_network_size; every
 * array [n_nodes] except frac_fp_imp [n_lc_scenes][n_nodes]; link arrays
 * (length, slope, a_floodplain, frac_fp_imp) valid for links 1..n_links,
 * from_n/to_n/net_perm/r_order as L11_fromN/L11_toN/L11_netPerm/L11_rOrder
 * (1-based; -9999 past the links), fdir11 packed over the L11 mask,
 * cell_row11/cell_col11 the L11 cells' grid coordinates, row_out/col_out
 * each L11 cell's outlet cell on the L0 grid (L11_rowOut / L11_colOut).
 * Any pointer may be NULL. */
typedef struct mhm_l11_network_out {
    int32_t n_nodes, n_outlets, n_links, nrows11, ncols11, n_l0_outlets;
    int32_t *fdir11, *cell_row11, *cell_col11, *from_n, *to_n, *net_perm, *r_order, *row_out, *col_out;
    double *length, *slope, *a_floodplain, *frac_fp_imp;
} mhm_l11_network_out;
int mhm_l11_network_size(int32_t nrows0, int32_t ncols0, const uint8_t *mask0, int32_t factor, int32_t *n_nodes);
int mhm_l11_network(const mhm_l0_flow *in, mhm_l11_network_out *out);
/* L11_L1_mapping (src/mRM/mo_mrm_net_startup.f90:61-226): for the L1 and
 * L11 grids at factors factor1 and factor11 of the L0 grid (integer
 * multiples of each other; sizes from mhm_l11_network_size with each
 * factor), L1_L11_Id [L1 cells] (the L11 cell containing each L1 cell) and
 * L11_L1_Id [L11 cells] (when L11 is finer), -9999 otherwise. */
int mhm_l1_l11_mapping(int32_t nrows0, int32_t ncols0, const uint8_t *mask0, int32_t factor1, int32_t factor11,
                       int32_t *l1_l11_id, int32_t *l11_l1_id);

/* Routing order of an L11 network (host computation, no device needed):
 * replaces L11_routing_order (src/mRM/mo_mrm_net_startup.f90:728-886) with an
 * O(nLinks x sweeps) algorithm giving the same ranks.  Inputs fromN/toN
 * [n_nodes] (1-based, links 1..n_nodes-n_outlets valid); outputs net_perm and
 * r_order [n_nodes] (entries past nLinks set to -9999 as in the reference). */
int mhm_routing_order(int32_t n_nodes, int32_t n_outlets, const int32_t *from_n, const int32_t *to_n,
                      int32_t *net_perm, int32_t *r_order);

/* Calendar of model steps tt0 .. tt0+n-1 of a run starting at Julian day
 * number jul_start (host computation): month (1-12), hour (0-23) and day of
 * year, as do_time_step obtains them from dec2date(newTime - 0.5)
 * (src/mHM/mo_mhm_interface_run.f90:355-363, src/common/
 * mo_common_datetime_type.f90:71-125).  Any output pointer may be NULL. */
int mhm_step_calendar(int32_t jul_start, int32_t timestep, int32_t tt0, int32_t n, int32_t *month,
                      int32_t *hour, int32_t *doy);
/* iLAI of steps tt0 .. tt0+n-1 for timeStep_LAI_input lai_mode (the month
 * for 0 / 1; the day / month / year count from the run's first step for
 * -1 / -2 / -3), as the cell chain reads its LAI-indexed parameters. */
int mhm_step_lai(int32_t jul_start, int32_t timestep, int32_t lai_mode, int32_t tt0, int32_t n, int32_t *lai);

/* ---- multiscale parameter regionalisation (MPR) ---- */

/* Level-0 inputs of mpr() for one basin and one land-cover scene, with the
 * classical soil database (iFlag_soilDB = 0): the arguments of
 * src/MPR/mo_multi_param_reg.f90:67-250 and of the start-up routines
 * generate_soil_database (src/MPR/mo_soil_database.f90:387-518) and
 * L0_variable_init (src/MPR/mo_mpr_startup.f90:237-337).  L0 cell arrays are
 * packed column-major over mask0 like the reference's level-0 arrays; all
 * class ids are 1-based.  Slope, aspect and LAI are taken as read_data leaves
 * them (src/MPR/mo_read_wrapper.f90:282-283, 335-336: slope >= 0.01,
 * aspect >= 1, LAI within [1e-10, 30]). */
typedef struct {
    int32_t n_cells0;          /* level0%nCells                                  */
    int32_t nrows0, ncols0;    /* level0 grid                                    */
    int32_t n_soil_types;      /* nSoilTypes                                     */
    int32_t max_soil_hor;      /* row stride of the per-soil horizon arrays      */
    int32_t n_geo_units;       /* nGeoUnits                                      */
    int32_t n_lai_classes;     /* > 0: LAI from a look-up table by class;
                                  0: gridded LAI0 [n_lai_steps][n_cells0]        */
    int32_t n_lai_steps;       /* entries of gridded LAI0 (0: 12 monthly slots);
                                  a context with a gridded LAI series
                                  (mhm_set_lai_series) needs its n_lai entries,
                                  and mhm_mpr then writes the LAI-indexed
                                  parameters into the series                     */
    double frac_sealed_city;   /* fracSealed_cityArea (mhm.nml)                  */
    const double *horizon_depth;  /* [n_horizons] HorizonDepth_mHM [mm]; the last
                                     entry is replaced per soil type by RZdepth  */
    const uint8_t *mask0;      /* [ncols0][nrows0] column-major, 1 inside        */
    const int32_t *l1_up, *l1_down, *l1_left, *l1_right; /* [n_cells] 1-based L0
                                  row/column bounds of each L1 cell (mo_grid.f90) */
    const int32_t *l1_nsub;    /* [n_cells] L0 cells inside each L1 cell         */
    const int32_t *soil_id0;   /* [n_cells0] L0_soilId                           */
    const int32_t *lcover0;    /* [n_cells0] L0_LCover (1 forest, 2 sealed, 3 pervious) */
    const int32_t *geo_unit0;  /* [n_cells0] L0_geoUnit                          */
    const double *slope0;      /* [n_cells0] L0_slope (its ranks give slope_emp) */
    const double *aspect0;     /* [n_cells0] L0_asp [deg]                        */
    const double *y0;          /* [n_cells0] L0 latitude (sign: hemisphere)      */
    const int32_t *lai_class0; /* [n_cells0] LAI class, n_lai_classes > 0        */
    const double *lai_lut;     /* [n_lai_classes][12] monthly LAI by class       */
    const double *lai0;        /* [n_lai_steps][n_cells0] gridded LAI, n_lai_classes == 0 */
    const int32_t *soil_n_hor;   /* [n_soil_types] soilDB%nHorizons              */
    const int32_t *soil_n_till;  /* [n_soil_types] soilDB%nTillHorizons          */
    const double *soil_ud, *soil_ld;   /* [n_soil_types][max_soil_hor] [mm]      */
    const double *soil_sand, *soil_clay, *soil_dbm; /* [n_soil_types][max_soil_hor] */
    const double *soil_rz_depth; /* [n_soil_types] soilDB%RZdepth [mm]           */
    const int32_t *geo_unit_list; /* [n_geo_units] GeoUnitList                   */
    const int32_t *geo_unit_kar;  /* [n_geo_units] GeoUnitKar (1: karstic)       */
} mhm_l0_desc;

/* Start-up of MPR for the context's basin: soil horizon weights Wd
 * (generate_soil_database), the empirical slope distribution slope_emp
 * (L0_variable_init), the land-cover and karst fractions of each L1 cell
 * (L0_fractionalCover_in_Lx, src/MPR/mo_upscaling_operators.f90:152-227) and
 * the device copy of the L0 maps in L1-block order.  Errors where the
 * reference stops: horizon depths outside a soil type, weights not summing
 * to 1, class ids out of range. */
int mhm_mpr_setup(mhm_ctx *ctx, const mhm_l0_desc *l0);

/* Start index (0-based) of each process's parameters in the global parameter
 * vector, processMatrix(:, 3) - processMatrix(:, 2) of
 * src/MPR/mo_mpr_read_config.f90:390-990: offsets[0..9] for processes 1..10,
 * offsets[10] = total length. */
int mhm_gamma_layout(int32_t proc_soilmoist, int32_t proc_pet, int32_t proc_routing, int32_t n_geo_units,
                     int32_t *offsets);

/* mpr() (src/MPR/mo_multi_param_reg.f90:67-654) for members member0 ..
 * member0+n-1 from their global parameter vectors gammas[n][n_gamma] (host),
 * evaluated on the device straight into the members' effective parameters;
 * with routing on, also reg_rout (src/mRM/mo_mrm_mpr.f90:61-119) from the
 * routing block of each vector.  Requires mhm_mpr_setup. */
int mhm_mpr(mhm_ctx *ctx, int32_t member0, int32_t n, const double *gammas, int32_t n_gamma);

/* mhm_mpr for one member that allocates no device memory: the parameter
 * vector and the soil tables live in a static device scratch of 65,536
 * doubles (512 KiB).  No counterpart in the reference (its mpr() allocates
 * Fortran temporaries on the host); it exists for callers that size device
 * memory once and must not cudaMalloc/cudaFree afterwards.  Returns
 * MHM_ERR_INVALID when the member needs more scratch than that (many soil
 * types or horizons; use mhm_mpr).  The scratch is shared per device:
 * overlapping calls race.  The first call on a device looks the scratch up
 * (cudaGetSymbolAddress) and must come before any stream capture starts on
 * that device.  Synchronises the context's stream before returning. */
int mhm_mpr_noalloc(mhm_ctx *ctx, int32_t member, const double *gamma, int32_t n_gamma);

/* The two parameter-independent start-up steps of mhm_mpr_setup as host
 * utilities (no device needed): soil horizon weights Wd [n_soil][n_h]
 * [max_hor] of generate_soil_database (src/MPR/mo_soil_database.f90:387-518;
 * horizon_depth[n_h-1] is overwritten as there), and the empirical slope
 * distribution of L0_variable_init (src/MPR/mo_mpr_startup.f90:237-337). */
int mhm_soil_weights(int32_t n_soil, int32_t max_hor, const int32_t *n_hor, const double *ud, const double *ld,
                     const double *rz_depth, int32_t n_h, double *horizon_depth, double *wd);
int mhm_slope_emp(int32_t n, const double *slope, double *slope_emp);

/* Start-up products of mhm_mpr_setup, for checking: "Wd" [n_soil_types]
 * [n_horizons][max_soil_hor], "slope_emp" [n_cells0], "horizon_depth"
 * [n_horizons] (after the RZdepth overwrite). */
int mhm_mpr_get_aux(mhm_ctx *ctx, const char *name, double *out);

/* Pinned host memory for forcing and outputs. */
int mhm_host_alloc(size_t bytes, void **ptr);
int mhm_host_free(void *ptr);

/* Build information: sm arch, number of kernels launched so far. */
int mhm_version(int32_t *major, int32_t *minor);
int64_t mhm_kernel_launch_count(void);

/* Elementary-function check: evaluates hmath log/exp/pow of n inputs on the
 * device (where == 1) or the host (where == 0): op 0 log(x), 1 exp(x),
 * 2 pow(x, y), 3 x / y.  Used by the tests to show host and device
 * bit-equality. */
int mhm_hmath_eval(int32_t op, int32_t where, int64_t n, const double *x, const double *y, double *out);

/* FP64 issue-rate probe: dependent DFMA chains on every SM for `iters`
 * iterations; returns achieved FP64 FLOP/s (2 per DFMA) in *flops. */
int mhm_probe_fp64(int64_t iters, double *flops);

#ifdef __cplusplus
}
#endif
#endif
