// engine.cu -- the C ABI of include/mhm_gpu.h: context, device memory, the
// chunked time loop (cell chain -> L1->L11 accumulation -> level routing) and
// state/variable access.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "fp64i.h"
#include "hmath.h"
#include "mhm_gpu.h"
#include "mhm_kernels.cuh"
#include "bounds.cuh"
#include "calendar.h"
#include "mpr_host.h"
#include "network.h"

namespace mhm {
cudaError_t launch_cell_chain(const CellArgs &a, int H, int occ, cudaStream_t s);
cudaError_t launch_steps_fill(StepInfo *steps, int64_t tt0, int32_t n, int32_t jul_start, int32_t timestep,
                              int32_t stride, int32_t lai_mode, cudaStream_t s);
cudaError_t launch_runoff_acc(const AccArgs &a, cudaStream_t s);
cudaError_t launch_route_tick(const RouteArgs &a, cudaStream_t s);
cudaError_t launch_route_walk(const RouteArgs &a, const RouteWalk &w, int cs, cudaStream_t s);
cudaError_t launch_qmod_step(const QmodStepArgs &a, cudaStream_t s);
cudaError_t launch_gauge_gather(const GaugeArgs &a, cudaStream_t s);
cudaError_t launch_qrouted(const QroutArgs &a, cudaStream_t s);
cudaError_t launch_reg_rout(int n_links, const double *p5, double ss_max, double TS, const double *length,
                            const double *slope, const double *ffp, const int32_t *link_pos, double *C1,
                            double *C2, cudaStream_t s);
cudaError_t launch_hmath_eval(int op, int64_t n, const double *x, const double *y, double *out, cudaStream_t s);
cudaError_t launch_fp64_probe(int64_t iters, int blocks, int threads, double *sink, cudaStream_t s);
cudaError_t launch_mpr(const MprArgs &a, cudaStream_t s);
cudaError_t launch_inflow(const InflowArgs &a, cudaStream_t s);
cudaError_t launch_cell_chain_fused(const FusedCellArgs &f, int hl, bool lean, int occ, cudaStream_t s);
cudaError_t launch_bc_selftest(cudaStream_t s);
// the bounds-checked build's status words, one per translation unit with checked kernels
cudaError_t bc_take_cell_chain(unsigned long long *out);
cudaError_t bc_take_cell_chain_o6(unsigned long long *out);
cudaError_t bc_take_cell_chain_o8(unsigned long long *out);
cudaError_t bc_take_routing(unsigned long long *out);
cudaError_t bc_take_mpr(unsigned long long *out);
} // namespace mhm

using namespace mhm;

namespace {

std::atomic<int64_t> g_launches{0};

template <class T>
struct DevBuf {
    T *p = nullptr;
    size_t n = 0;
    ~DevBuf() { release(); }
    void release()
    {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    cudaError_t ensure(size_t count)
    {
        if (count <= n && p) return cudaSuccess;
        release();
        if (count == 0) return cudaSuccess;
        cudaError_t e = cudaMalloc(&p, count * sizeof(T));
        if (e != cudaSuccess) {
            p = nullptr;
            return e;
        }
        n = count;
        return cudaSuccess;
    }
};

struct TimedLaunch {
    int kind;
    cudaEvent_t a, b;
};

// One aggregated output set (mHM's outputFlxState or mRM's Qrouted): the
// interval schedule, the host's view of the device counters after all
// enqueued work, and the device running sums / written intervals.
struct OutSet {
    bool on = false;
    int32_t interval = 0, max_slots = 0, n_planes = 0;
    int64_t warm = 0, n_tt = 0;
    int32_t slots = 0, cnt = 0;      // intervals written (not yet read), steps in the open interval
    std::vector<int64_t> slot_tt;    // model step that closed each written interval
    DevBuf<double> acc, out;
};

// The routing wavefront of one chunk (D + n_sub - 1 launches of
// route_tick_kernel) captured once as a CUDA graph per argument set and
// replayed for every chunk of that shape: the tick launches differ only in
// tick / position range, which depend on the network and the chunk length.
struct RouteGraph {
    RouteArgs key{};
    int32_t n_ticks = 0;
    cudaGraphExec_t exec = nullptr;
};

bool same_route_shape(const RouteArgs &a, const RouteArgs &b)
{
    return a.n_nodes == b.n_nodes && a.n_members == b.n_members && a.n_steps == b.n_steps && a.sub == b.sub &&
           a.rdiv == b.rdiv && a.n_qsteps == b.n_qsteps && a.pos_level == b.pos_level && a.up_ptr == b.up_ptr &&
           a.up_pos == b.up_pos && a.pos_flags == b.pos_flags && a.C1 == b.C1 && a.C2 == b.C2 && a.qout == b.qout &&
           a.qtr == b.qtr && a.qmod == b.qmod && a.qtin1 == b.qtin1 && a.qtr1 == b.qtr1 &&
           a.member_step0 == b.member_step0;
}

struct ForcingSrc {
    const double *ptr = nullptr;
    int32_t row0 = 0, n_rows = 0, on_device = 0;
    bool set = false;
};

} // namespace

struct mhm_ctx {
    // domain
    int32_t N = 0, H = 0, L = 0, n_out = 0, n_links = 0, M = 1, G = 0;
    int32_t timestep = 1, proc_sm = 1, proc_pet = 0, proc_rout = 1, ntfd = 24, jul_start = 0, map_flag = 1;
    int32_t read_states = 0;
    int device = 0;
    MonthTables tab{};
    double ss_max = 0.0;
    LevelNetwork net;
    std::vector<int32_t> gauge_pos;
    std::vector<int32_t> link_to;    // [n_links] 0-based node each link drains into
    DevBuf<int32_t> nonfinite;       // [M] per-member non-finite flags of the cell chain
    // inflow gauges: position and headwater flag of each, daily discharge
    int32_t n_inflow = 0, inflow_day0 = 1, inflow_ndays = 0;
    std::vector<int32_t> inflow_pos;
    std::vector<int8_t> inflow_hw;
    DevBuf<int32_t> inflow_pos_d;
    DevBuf<int8_t> inflow_hw_d;
    DevBuf<double> inflow_q;
    // device: static
    DevBuf<double> params, states, latitude, l1_area, pos_area, length, slope, ffp, rout_p5;
    DevBuf<double> C1, C2, qtin1, qtr1, qout_last, qmod_last;
    DevBuf<int32_t> node_cell_ptr, node_cells, pos_l11_l1, up_ptr, up_pos, link_pos, gauge_pos_d, pos_level;
    DevBuf<int8_t> pos_flags;
    // device: per run / chunk
    DevBuf<StepInfo> steps;
    DevBuf<double> tro[2], qout, qtr, qmod, q_gauge[2];
    DevBuf<double> stage[kForcKinds][2];
    int32_t tc_cap = 0, stage_rows = 0;
    size_t qg_cap[2] = {0, 0};
    int64_t chunk_seq = 0, call_seq = 0;
    bool slot_used[2] = {false, false};
    bool pending_outputs = false;
    // forcing
    ForcingSrc forc[kForcKinds];
    // gauge series of the calls in flight: device -> pinned staging (an
    // asynchronous copy; a copy into pageable memory would block the host
    // until the routing finished) -> the caller's buffer at the next
    // synchronisation point
    struct GaugeStage {
        double *pinned = nullptr;
        size_t cap = 0, bytes = 0;
        double *dst = nullptr;
        cudaEvent_t ev = nullptr;
        bool active = false;
    } qg_stage[2];
    // outputs
    int32_t out_tro = 0, out_qmod = 0, out_flux = 0;
    DevBuf<double> flux_d[2];
    // aggregated flux/state outputs and Qrouted
    OutSet fso, qro;
    int8_t fs_plane[kOutFlags + 1];
    uint64_t fs_avg = 0;
    DevBuf<int64_t> w_tt;
    DevBuf<double> w_fs, w_sms;
    std::vector<double> host_aet, host_loss;
    std::vector<double> host_tro, host_qmod;
    int32_t last_steps = 0;
    // execution
    cudaStream_t stream = nullptr, copy_stream = nullptr, route_stream = nullptr;
    cudaEvent_t ev_copied[2] = {nullptr, nullptr}, ev_consumed[2] = {nullptr, nullptr};
    cudaEvent_t ev_cell_done[2] = {nullptr, nullptr}, ev_acc_done[2] = {nullptr, nullptr};
    cudaEvent_t ev_route_end = nullptr, run_a = nullptr;
    cudaEvent_t ev_poll[3] = {nullptr, nullptr, nullptr};
    bool timing = false;
    std::vector<TimedLaunch> pending;
    int64_t t_launches[4] = {0, 0, 0, 0};
    double t_ms[4] = {0, 0, 0, 0};
    size_t chunk_bytes = (size_t)8 << 30;
    int32_t route_sub = 8; // steps per wavefront sub-chunk (4, 8 or 16)
    bool route_graphs_on = true;
    std::vector<RouteGraph> route_graphs; // most recently used last
    // 0: one launch per wavefront tick (replayed from a CUDA graph); 4, 8, 16:
    // the whole wavefront of a chunk in one launch of clusters of that many CTAs
    int32_t route_cluster = 0;
    DevBuf<int32_t> level_ptr_d;
    // timeStep_LAI_input: 0 monthly LAI slots; -1 / -2 / -3 a gridded LAI series
    // of n_lai entries, its parameters in lai_series [M][3][n_lai][N]
    int32_t lai_mode = 0, n_lai = 0;
    DevBuf<double> lai_series;
    int32_t cell_occ = 4;  // cell-chain register variant: resident blocks per SM (4, 6, 8)
    int32_t chunk_cap = 0; // most time steps per chunk (0: the device-memory budget decides)
    // routing case 2: per-member routing time step [s] and the link lengths
    std::vector<double> ts_rout, length_h;
    DevBuf<double> qmod_sub;
    // member mode (mhm_run_members_async) and device-resident state snapshots
    DevBuf<StepInfo> steps_all;
    int64_t steps_all_filled = 0;
    // per-call member table in a ring: a call may be enqueued while the
    // routing of earlier calls (on route_stream) still reads theirs
    DevBuf<int32_t> member_s0[4];
    cudaEvent_t ev_members_done[4] = {nullptr, nullptr, nullptr, nullptr};
    int64_t member_calls = 0;
    const int32_t *member_s0_cur = nullptr;
    std::vector<int32_t> member_s0_h;
    DevBuf<double> snap;
    int32_t n_snap = 0;
    // multiscale parameter regionalisation (after mhm_mpr_setup)
    bool mpr_ready = false;
    // read_meteo_weights: [3][24][12][N] (pre, pet, temp)
    DevBuf<double> meteo_w;
    bool meteo_w_on = false;
    MprSetup mpr;
    DevBuf<int32_t> mpr_nhor, mpr_ntill, mpr_nsub;
    DevBuf<uint32_t> mpr_code;
    DevBuf<double> mpr_soil, mpr_se, mpr_asp, mpr_lai, mpr_frac, mpr_lut, mpr_gamma, mpr_table, mpr_petlai;
    std::string err;
};

// A batch of contexts whose cell chains run in one persistent launch.
struct mhm_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev_done = nullptr, ev_staged = nullptr;
    bool staged = false;
    std::vector<cudaEvent_t> ev_pre;
    DevBuf<CellArgs> args;
    DevBuf<int32_t> tile_ctx, queue;
    DevBuf<int64_t> tile_item0;
    CellArgs *h_args = nullptr;
    int32_t *h_tile_ctx = nullptr;
    int64_t *h_item0 = nullptr;
    size_t cap_ctx = 0, cap_tiles = 0;
    int64_t rounds = 0, tiles_total = 0;
    int32_t occ = 8; // register variant of the fused launch: 4 or 8 resident blocks per SM
    std::string err;
};

namespace {

int fail(mhm_ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    return code;
}

int cuda_fail(mhm_ctx *c, cudaError_t e, const char *what)
{
    int code = (e == cudaErrorMemoryAllocation) ? MHM_ERR_OOM : MHM_ERR_CUDA;
    return fail(c, code, std::string(what) + ": " + cudaGetErrorString(e));
}

#define CK(call, what)                                                                                             \
    do {                                                                                                           \
        cudaError_t e_ = (call);                                                                                   \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what);                                                    \
    } while (0)

// Makes a device current for the lifetime of the guard and puts the calling
// thread's previous device back on exit, so that a context's allocations and
// launches land on its own GPU whatever device the caller has current, and
// the caller's own CUDA calls afterwards still see the device it chose.
struct DeviceGuard {
    int prev = -1;
    cudaError_t err = cudaSuccess;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) err = cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
    DeviceGuard(const DeviceGuard &) = delete;
    DeviceGuard &operator=(const DeviceGuard &) = delete;
};

// An NVTX range over a host phase (shown by Nsight Systems / ncu's NVTX
// filters; free when no tool is attached).
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// First statement of every context entry point that touches the GPU.
#define ON_CTX_DEVICE(ctx)                                                                                         \
    DeviceGuard dev_guard_((ctx)->device);                                                                         \
    if (dev_guard_.err != cudaSuccess) return cuda_fail(ctx, dev_guard_.err, "set device")

// Host replica of the device interval bookkeeping over steps tt_a .. tt_a+n-1
// (same calendar and writeout rule as the kernels); with `commit` the set's
// counters and closing steps advance, else only the written count is returned.
int32_t out_advance(OutSet &o, int32_t jul_start, int32_t timestep, int64_t tt_a, int64_t n, bool commit)
{
    int32_t cnt = o.cnt, wrote = 0;
    for (int64_t tt = tt_a; tt < tt_a + n; ++tt) {
        if (tt <= o.warm) continue;
        ++cnt;
        if (out_writeout(o.interval, tt - o.warm, tt, o.n_tt, step_dflags(jul_start, timestep, tt))) {
            ++wrote;
            cnt = 0;
            if (commit) o.slot_tt.push_back(tt);
        }
    }
    if (commit) {
        o.cnt = cnt;
        o.slots += wrote;
    }
    return wrote;
}

template <class T>
cudaError_t upload(DevBuf<T> &b, const T *host, size_t n, cudaStream_t s)
{
    cudaError_t e = b.ensure(n);
    if (e != cudaSuccess) return e;
    if (n == 0) return cudaSuccess;
    return cudaMemcpyAsync(b.p, host, n * sizeof(T), cudaMemcpyHostToDevice, s);
}

// Timed launch bracket: events recorded on the launching stream.
struct Bracket {
    mhm_ctx *c;
    int kind;
    cudaStream_t s;
    cudaEvent_t a = nullptr, b = nullptr;
    Bracket(mhm_ctx *cc, int k, cudaStream_t st) : c(cc), kind(k), s(st)
    {
        if (c->timing) {
            cudaEventCreate(&a);
            cudaEventCreate(&b);
            cudaEventRecord(a, s);
        }
    }
    void done()
    {
        if (c->timing) {
            cudaEventRecord(b, s);
            c->pending.push_back({kind, a, b});
        }
    }
};

// The routing stream gets the highest priority: its wavefront ticks are short,
// latency-bound launches that should take the next free SM slot ahead of the
// cell-chain blocks they overlap with.
cudaError_t route_stream_create(cudaStream_t *s)
{
    int lo = 0, hi = 0;
    if (cudaDeviceGetStreamPriorityRange(&lo, &hi) != cudaSuccess) hi = 0;
    return cudaStreamCreateWithPriority(s, cudaStreamNonBlocking, hi);
}

void harvest_timing(mhm_ctx *c)
{
    for (auto &t : c->pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, t.a, t.b) == cudaSuccess) {
            c->t_ms[t.kind] += ms;
            c->t_launches[t.kind] += 1;
        }
        cudaEventDestroy(t.a);
        cudaEventDestroy(t.b);
    }
    c->pending.clear();
}

} // namespace

// Scratch of mhm_mpr_noalloc: the parameter vector, the soil table and the
// LAI-correction table of one member, in one statically sized device array
// so that the call needs no device allocation.  65,536 doubles = 512 KiB.
constexpr size_t kMprScratchDoubles = 65536;
static __device__ __align__(256) double g_mpr_scratch[kMprScratchDoubles];
// its address on each device, looked up on first use
constexpr int kMaxScratchDevices = 64;
static std::mutex g_scratch_mu;
static double *g_scratch_addr[kMaxScratchDevices] = {};
static inline size_t align32(size_t n) { return (n + 31) & ~(size_t)31; } // 256-byte steps

namespace {

// processMatrix(:, 2) of src/MPR/mo_mpr_read_config.f90:390-990 (and the
// routing block set there for mRM), accumulated into start offsets
// Routing time steps [s] the adaptive routing can choose
// (src/mRM/mo_mrm_constants.F90:42-46)
constexpr double kGivenTS[19] = {60.0,    120.0,   180.0,   240.0,   300.0,   360.0,   600.0,
                                 720.0,   900.0,   1200.0,  1800.0,  3600.0,  7200.0,  10800.0,
                                 14400.0, 21600.0, 28800.0, 43200.0, 86400.0};

// FORCES locate (in-tree copy pre-proc/mtCLIM/mo_utils.f90:1329-1346): index
// (1-based) of the nearest table value, minus one when it lies above y (LE
// with relative-epsilon equality)
int locate_ts(double y)
{
    int c = 0;
    double best = std::fabs(kGivenTS[0] - y);
    for (int i = 1; i < 19; ++i)
        if (std::fabs(kGivenTS[i] - y) < best) {
            best = std::fabs(kGivenTS[i] - y);
            c = i;
        }
    const double a = kGivenTS[c], eps = 2.220446049250313e-16;
    const bool le = !(((eps * std::fabs(y) - std::fabs(a - y)) < 0.0) && (a > y));
    return le ? c + 1 : c;
}

} // namespace

// Routing case 2 for one member (mrm_update_param, src/mRM/mo_mrm_mpr.f90:
// 241-329): K = length / celerity per link, TSrout from the smallest K,
// Muskingum coefficients with xi = 0 (written at the links' positions).
// mrm_update_param (src/mRM/mo_mrm_mpr.f90:241-329): K = length / celerity
// per link -- one celerity for routing case 2, the link's own (L11_celerity)
// for case 3 -- the routing step from the shortest K, C1/C2 with xi = 0.
static int set_adaptive_member(mhm_ctx *ctx, int32_t m, double celerity, const double *link_celerity)
{
    const size_t L = ctx->L;
    const int nl = ctx->n_links;
    if (nl == 0) return MHM_OK;
    auto cel = [&](int i) { return link_celerity ? link_celerity[i] : celerity; };
    for (int i = 0; i < nl; ++i)
        if (!(cel(i) > 0.0)) return fail(ctx, MHM_ERR_INVALID, "streamflow celerity must be positive");
    const double xi = std::fabs(0.0); // rout_space_weight
    double kmin = HUGE_VAL;
    for (int i = 0; i < nl; ++i) kmin = std::min(kmin, ctx->length_h[i] / cel(i));
    int ind = locate_ts(kmin);
    if (ind < 1) ind = 1;
    const double ts = kGivenTS[ind - 1];
    std::vector<double> c1(L, 0.0), c2(L, 0.0);
    for (int i = 0; i < nl; ++i) {
        const double K = ctx->length_h[i] / cel(i);
        const double a = ts / (K * (1.0 - xi) + 0.5 * ts);
        c1[ctx->net.link_pos[i]] = a;
        c2[ctx->net.link_pos[i]] = 1.0 - a * K / ts;
    }
    CK(cudaMemcpyAsync(ctx->C1.p + m * L, c1.data(), L * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "C1");
    CK(cudaMemcpyAsync(ctx->C2.p + m * L, c2.data(), L * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "C2");
    CK(cudaStreamSynchronize(ctx->stream), "C1/C2 sync");
    ctx->ts_rout[m] = ts;
    return MHM_OK;
}

namespace {

bool gamma_layout(int32_t proc_sm, int32_t proc_pet, int32_t proc_rout, int32_t n_geo, GammaOffsets &o)
{
    int32_t n_sm, n_pet, n_rout;
    switch (proc_sm) {
    case 1: n_sm = 17; break;
    case 2: n_sm = 18; break;
    case 3: n_sm = 22; break;
    case 4: n_sm = 21; break;
    default: return false;
    }
    switch (proc_pet) {
    case -1: n_pet = 5; break;
    case 0: n_pet = 3; break;
    case 1: n_pet = 4; break;
    case 2: n_pet = 2; break;
    case 3: n_pet = 7; break;
    default: return false;
    }
    switch (proc_rout) {
    case 0: n_rout = 0; break;
    case 1: n_rout = 5; break;
    case 2:
    case 3: n_rout = 1; break;
    default: return false;
    }
    if (n_geo < 0) return false;
    o.interc = 0;
    o.snow = o.interc + 1;
    o.soil = o.snow + 8;
    o.runoff = o.soil + n_sm;
    o.pet = o.runoff + 1;
    o.interflow = o.pet + n_pet;
    o.perc = o.interflow + 5;
    o.routing = o.perc + 3;
    o.geo = o.routing + n_rout;
    o.total = o.geo + n_geo; // neutron process 10 off: no parameters
    o.n_soil_params = n_sm;
    return true;
}

} // namespace

namespace {
// Copies the written intervals to the caller and frees the device slots.
int read_outset(mhm_ctx *ctx, OutSet &o, double *out, int64_t *slot_tt, int32_t max_slots, int32_t *n_slots,
                bool by_node)
{
    if (!o.on) return fail(ctx, MHM_ERR_INVALID, "these outputs are not enabled");
    if (int rc = mhm_sync(ctx)) return rc;
    if (n_slots) *n_slots = o.slots;
    if (!out) return MHM_OK; // query only
    if (o.slots > max_slots) return fail(ctx, MHM_ERR_INVALID, "buffer holds fewer intervals than were written");
    const size_t per = (size_t)o.n_planes * ctx->M * (by_node ? (size_t)ctx->L : (size_t)ctx->N);
    if (o.slots > 0)
        CK(cudaMemcpy(out, o.out.p, (size_t)o.slots * per * sizeof(double), cudaMemcpyDeviceToHost), "outputs");
    if (by_node) { // routing-level positions -> L11 node order
        const size_t L = ctx->L;
        std::vector<double> row(L);
        for (size_t r = 0; r < (size_t)o.slots * ctx->M; ++r) {
            double *q = out + r * L;
            for (size_t v = 0; v < L; ++v) row[v] = q[ctx->net.pos_of_node[v]];
            std::memcpy(q, row.data(), L * sizeof(double));
        }
    }
    if (slot_tt)
        for (int32_t i = 0; i < o.slots; ++i) slot_tt[i] = o.slot_tt[i];
    o.slots = 0;
    o.slot_tt.clear();
    return MHM_OK;
}
} // namespace

extern "C" {

int mhm_version(int32_t *major, int32_t *minor)
{
    if (major) *major = 0;
    if (minor) *minor = 1;
    return MHM_OK;
}

int64_t mhm_kernel_launch_count(void) { return g_launches.load(); }

const char *mhm_last_error(const mhm_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

void *mhm_ctx_stream(mhm_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int mhm_ctx_create(const mhm_domain_desc *d, int32_t device, mhm_ctx **out)
{
    NvtxRange nvtx_("mhm: context create");
    if (!d || !out) return MHM_ERR_INVALID;
    *out = nullptr;
    mhm_ctx *ctx = new mhm_ctx();
    auto bad = [&](const std::string &m) {
        std::string msg = m;
        delete ctx;
        std::fprintf(stderr, "mhm_ctx_create: %s\n", msg.c_str());
        return MHM_ERR_INVALID;
    };
    if (d->n_cells < 1) return bad("n_cells < 1");
    if (d->n_horizons < 1 || d->n_horizons > kMaxHorizons) return bad("n_horizons must be 1..8");
    if (d->n_members < 1) return bad("n_members < 1");
    if (d->timestep < 1 || 24 % d->timestep != 0) return bad("timestep must divide 24 hours");
    if (d->proc_soilmoist < 1 || d->proc_soilmoist > 4) return bad("proc_soilmoist must be 1..4");
    if (d->proc_pet < -1 || d->proc_pet > 3) return bad("proc_pet must be -1, 0, 1, 2 or 3");
    if (d->proc_routing < 0 || d->proc_routing > 3) return bad("proc_routing must be 0, 1, 2 or 3");
    if (d->n_tstep_forcing_day != 24 && d->n_tstep_forcing_day != 1)
        return bad("n_tstep_forcing_day must be 24 or 1");
    if (d->jul_start < 2299161) return bad("jul_start before the Gregorian reform is not supported");
    if (!d->evap_coeff) return bad("evap_coeff missing");
    if (d->n_tstep_forcing_day == 1 && (!d->fday_prec || !d->fnight_prec || !d->fday_pet || !d->fnight_pet ||
                                        !d->fday_temp || !d->fnight_temp))
        return bad("day/night ratios missing for daily forcing");
    if (d->proc_pet == 1 && !d->latitude) return bad("latitude missing for Hargreaves PET");
    ctx->N = d->n_cells;
    ctx->H = d->n_horizons;
    ctx->M = d->n_members;
    ctx->timestep = d->timestep;
    ctx->proc_sm = d->proc_soilmoist;
    ctx->proc_pet = d->proc_pet;
    ctx->proc_rout = d->proc_routing;
    ctx->ntfd = d->n_tstep_forcing_day;
    ctx->jul_start = d->jul_start;
    ctx->map_flag = d->map_flag;
    ctx->read_states = d->read_states;
    for (int i = 0; i < 12; ++i) {
        ctx->tab.evap[i] = d->evap_coeff[i];
        if (d->n_tstep_forcing_day == 1) {
            ctx->tab.fday_prec[i] = d->fday_prec[i];
            ctx->tab.fnight_prec[i] = d->fnight_prec[i];
            ctx->tab.fday_pet[i] = d->fday_pet[i];
            ctx->tab.fnight_pet[i] = d->fnight_pet[i];
            ctx->tab.fday_temp[i] = d->fday_temp[i];
            ctx->tab.fnight_temp[i] = d->fnight_temp[i];
        }
    }
    if (ctx->proc_rout >= 1) {
        if (d->n_nodes < 1 || !d->l1_l11_id || !d->net_perm || !d->from_n || !d->to_n)
            return bad("routing arrays missing");
        if (!d->map_flag && (!d->l11_l1_id || !d->l11_area_km2)) return bad("L11_L1_Id/areas missing");
        if (d->map_flag && !d->l1_area_km2) return bad("L1 cell areas missing");
        ctx->L = d->n_nodes;
        ctx->n_out = d->n_outlets;
        std::string err;
        if (ctx->L > 1) {
            if (!build_level_network(d->n_nodes, d->n_outlets, d->net_perm, d->from_n, d->to_n, ctx->net, err))
                return bad(err);
        } else {
            ctx->net = LevelNetwork{};
            ctx->net.n_nodes = 1;
            ctx->net.n_levels = 1;
            ctx->net.level_ptr = {0, 1};
            ctx->net.pos_of_node = {0};
            ctx->net.node_of_pos = {0};
            ctx->net.up_ptr = {0, 0};
            ctx->net.pos_flags = {2}; // Qmod = qOUT for a single node
        }
        ctx->n_links = ctx->net.n_links;
        for (int i = 0; i < ctx->n_links; ++i) ctx->link_to.push_back(d->to_n[i] - 1);
        if (ctx->n_links > 0 && (!d->length || !d->slope || !d->ffp_imp)) return bad("link length/slope/fFPimp missing");
        ctx->G = d->n_gauges;
        if (ctx->G < 0 || (ctx->G > 0 && !d->gauge_node)) return bad("gauges");
        for (int g = 0; g < ctx->G; ++g) {
            int v = d->gauge_node[g] - 1;
            if (v < 0 || v >= ctx->L) return bad("gauge node out of range");
            ctx->gauge_pos.push_back(ctx->net.pos_of_node[v]);
        }
        for (int k = 0; k < ctx->N; ++k)
            if (d->l1_l11_id[k] < 1 || d->l1_l11_id[k] > ctx->L) return bad("L1_L11_Id out of range");
        if (!d->map_flag)
            for (int i = 0; i < ctx->L; ++i)
                if (d->l11_l1_id[i] < 1 || d->l11_l1_id[i] > ctx->N) return bad("L11_L1_Id out of range");
    }
    // device
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) {
        delete ctx;
        std::fprintf(stderr, "mhm_ctx_create: no CUDA device (%s)\n", cudaGetErrorString(e));
        return MHM_ERR_CUDA;
    }
    if (device >= ndev) return bad("device index out of range");
    int cur_dev = 0;
    if (device < 0 && cudaGetDevice(&cur_dev) != cudaSuccess) cur_dev = 0;
    ctx->device = device >= 0 ? device : cur_dev;
    // the context's buffers and streams live on ctx->device; the caller's
    // current device is put back on return
    DeviceGuard dg(ctx->device);
    if (dg.err != cudaSuccess) return bad(std::string("cannot use device: ") + cudaGetErrorString(dg.err));
    auto ck = [&](cudaError_t ee, const char *w) {
        if (ee != cudaSuccess) {
            std::fprintf(stderr, "mhm_ctx_create: %s: %s\n", w, cudaGetErrorString(ee));
            return false;
        }
        return true;
    };
    if (!ck(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking), "stream") ||
        !ck(cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking), "copy stream") ||
        !ck(route_stream_create(&ctx->route_stream), "route stream")) {
        mhm_ctx_destroy(ctx);
        return MHM_ERR_CUDA;
    }
    for (int i = 0; i < 2; ++i) {
        cudaEventCreateWithFlags(&ctx->ev_copied[i], cudaEventDisableTiming);
        cudaEventCreateWithFlags(&ctx->ev_consumed[i], cudaEventDisableTiming);
        cudaEventCreateWithFlags(&ctx->ev_cell_done[i], cudaEventDisableTiming);
        cudaEventCreateWithFlags(&ctx->ev_acc_done[i], cudaEventDisableTiming);
    }
    cudaEventCreateWithFlags(&ctx->ev_route_end, cudaEventDisableTiming);
    const size_t N = ctx->N, M = ctx->M, H = ctx->H, L = ctx->L;
    bool ok = true;
    ok = ok && ck(ctx->params.ensure(M * n_param_planes((int)H) * N), "params");
    ok = ok && ck(ctx->states.ensure(M * n_state_planes((int)H) * N), "states");
    ok = ok && ck(ctx->nonfinite.ensure(M), "member flags");
    if (ok) cudaMemsetAsync(ctx->nonfinite.p, 0, M * sizeof(int32_t), ctx->stream);
    if (ok) {
        cudaMemsetAsync(ctx->params.p, 0, ctx->params.n * sizeof(double), ctx->stream);
        cudaMemsetAsync(ctx->states.p, 0, ctx->states.n * sizeof(double), ctx->stream);
    }
    if (ok && ctx->proc_pet == 1) ok = ck(upload(ctx->latitude, d->latitude, N, ctx->stream), "latitude");
    if (ok && ctx->proc_rout >= 1) {
        const LevelNetwork &net = ctx->net;
        // L1 cells of each node in ascending cell order, by position
        std::vector<int32_t> cnt(L + 1, 0), cells(N);
        for (size_t k = 0; k < N; ++k) cnt[net.pos_of_node[d->l1_l11_id[k] - 1] + 1]++;
        for (size_t p = 0; p < L; ++p) cnt[p + 1] += cnt[p];
        std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
        for (size_t k = 0; k < N; ++k) cells[fill[net.pos_of_node[d->l1_l11_id[k] - 1]]++] = (int32_t)k;
        std::vector<int32_t> pl1(L, 0);
        std::vector<double> parea(L, 0.0);
        for (size_t p = 0; p < L; ++p) {
            int v = net.node_of_pos[p];
            if (!d->map_flag) pl1[p] = d->l11_l1_id[v] - 1;
            parea[p] = d->l11_area_km2 ? d->l11_area_km2[v] : 0.0;
        }
        ok = ok && ck(upload(ctx->node_cell_ptr, cnt.data(), L + 1, ctx->stream), "cell ptr");
        ok = ok && ck(upload(ctx->node_cells, cells.data(), N, ctx->stream), "cells");
        ok = ok && ck(upload(ctx->pos_l11_l1, pl1.data(), L, ctx->stream), "l11_l1");
        ok = ok && ck(upload(ctx->pos_area, parea.data(), L, ctx->stream), "l11 area");
        if (d->map_flag) ok = ok && ck(upload(ctx->l1_area, d->l1_area_km2, N, ctx->stream), "l1 area");
        std::vector<int32_t> plev(L, 0);
        for (int l = 0; l < net.n_levels; ++l)
            for (int p = net.level_ptr[l]; p < net.level_ptr[l + 1]; ++p) plev[p] = l;
        ok = ok && ck(upload(ctx->pos_level, plev.data(), L, ctx->stream), "levels");
        ok = ok && ck(upload(ctx->level_ptr_d, net.level_ptr.data(), net.level_ptr.size(), ctx->stream), "level ptr");
        ok = ok && ck(upload(ctx->up_ptr, net.up_ptr.data(), L + 1, ctx->stream), "up ptr");
        ok = ok && ck(upload(ctx->up_pos, net.up_pos.data(), net.up_pos.size(), ctx->stream), "up pos");
        ok = ok && ck(upload(ctx->pos_flags, net.pos_flags.data(), L, ctx->stream), "flags");
        ok = ok && ck(upload(ctx->link_pos, net.link_pos.data(), net.link_pos.size(), ctx->stream), "link pos");
        ok = ok && ck(upload(ctx->gauge_pos_d, ctx->gauge_pos.data(), ctx->gauge_pos.size(), ctx->stream), "gauges");
        if (ctx->n_links > 0) {
            ok = ok && ck(upload(ctx->length, d->length, ctx->n_links, ctx->stream), "length");
            ok = ok && ck(upload(ctx->slope, d->slope, ctx->n_links, ctx->stream), "slope");
            ok = ok && ck(upload(ctx->ffp, d->ffp_imp, ctx->n_links, ctx->stream), "ffp");
            double mx = -HUGE_VAL;
            for (int i = 0; i < ctx->n_links; ++i) mx = std::max(mx, d->slope[i]);
            ctx->ss_max = mx;
        }
        ok = ok && ck(ctx->rout_p5.ensure(5 * M), "p5");
        ctx->ts_rout.assign(M, 0.0);
        if (ctx->n_links > 0) ctx->length_h.assign(d->length, d->length + ctx->n_links);
        for (auto *b : {&ctx->C1, &ctx->C2, &ctx->qtin1, &ctx->qtr1, &ctx->qout_last, &ctx->qmod_last}) {
            ok = ok && ck(b->ensure(M * L), "routing state");
            if (ok) cudaMemsetAsync(b->p, 0, M * L * sizeof(double), ctx->stream);
        }
    }
    if (ok) ok = ck(cudaStreamSynchronize(ctx->stream), "init sync");
    if (!ok) {
        mhm_ctx_destroy(ctx);
        return MHM_ERR_OOM;
    }
    if (const char *s = std::getenv("MHM_CHUNK_BYTES")) ctx->chunk_bytes = (size_t)std::atoll(s);
    if (const char *s = std::getenv("MHM_ROUTE_SUB")) {
        int v = std::atoi(s);
        if (v >= 1 && v <= 16) ctx->route_sub = v;
    }
    if (const char *s = std::getenv("MHM_CELL_OCC")) {
        int v = std::atoi(s);
        if (v == 4 || v == 6 || v == 8) ctx->cell_occ = v;
    }
    if (const char *s = std::getenv("MHM_ROUTE_GRAPH")) ctx->route_graphs_on = std::atoi(s) != 0;
    if (const char *s = std::getenv("MHM_ROUTE_CLUSTER")) {
        int v = std::atoi(s);
        if (v == 0 || v == 4 || v == 8 || v == 16) ctx->route_cluster = v;
    }
    *out = ctx;
    return MHM_OK;
}

int mhm_ctx_destroy(mhm_ctx *ctx)
{
    if (!ctx) return MHM_OK;
    DeviceGuard dg(ctx->device); // release everything on the context's own device
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
    if (ctx->route_stream) cudaStreamSynchronize(ctx->route_stream);
    harvest_timing(ctx);
    for (int i = 0; i < 2; ++i) {
        if (ctx->ev_copied[i]) cudaEventDestroy(ctx->ev_copied[i]);
        if (ctx->ev_consumed[i]) cudaEventDestroy(ctx->ev_consumed[i]);
        if (ctx->ev_cell_done[i]) cudaEventDestroy(ctx->ev_cell_done[i]);
        if (ctx->ev_acc_done[i]) cudaEventDestroy(ctx->ev_acc_done[i]);
    }
    if (ctx->ev_route_end) cudaEventDestroy(ctx->ev_route_end);
    for (cudaEvent_t e : ctx->ev_poll)
        if (e) cudaEventDestroy(e);
    for (auto &st : ctx->qg_stage) {
        if (st.pinned) cudaFreeHost(st.pinned);
        if (st.ev) cudaEventDestroy(st.ev);
    }
    for (cudaEvent_t e : ctx->ev_members_done)
        if (e) cudaEventDestroy(e);
    if (ctx->run_a) cudaEventDestroy(ctx->run_a);
    for (auto &rg : ctx->route_graphs)
        if (rg.exec) cudaGraphExecDestroy(rg.exec);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    if (ctx->route_stream) cudaStreamDestroy(ctx->route_stream);
    delete ctx;
    return MHM_OK;
}

int mhm_set_eff_params(mhm_ctx *ctx, int32_t m, const mhm_eff_params *p)
{
    if (!ctx || !p) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc; // no enqueued step may still read what changes
    if (m < 0 || m >= ctx->M) return fail(ctx, MHM_ERR_INVALID, "member out of range");
    const size_t N = ctx->N;
    const int H = ctx->H, np = n_param_planes(H);
    const double *scalars[16] = {p->fSealed,   p->alpha,     p->degDayInc, p->degDayMax,   p->degDayNoPre,
                                 p->fAsp,      p->HarSamCoeff, p->karstLoss, p->kFastFlow, p->kSlowFlow,
                                 p->kBaseFlow, p->kPerco,    p->jarvis_thresh_c1, p->tempThresh, p->unsatThresh,
                                 p->sealedThresh};
    double *base = ctx->params.p + (size_t)m * np * N;
    for (int i = 0; i < 16; ++i) {
        if (!scalars[i]) {
            if (i == P_HARSAM && ctx->proc_pet != 1) continue;
            if (i == P_FASP && ctx->proc_pet == -1) continue;
            if (i == P_JARVIS && (ctx->proc_sm == 1 || ctx->proc_sm == 4)) continue;
            return fail(ctx, MHM_ERR_INVALID, "effective parameter " + std::to_string(i) + " missing");
        }
        CK(cudaMemcpyAsync(base + (size_t)i * N, scalars[i], N * sizeof(double), cudaMemcpyHostToDevice,
                           ctx->stream),
           "params");
    }
    if (!p->maxInter) return fail(ctx, MHM_ERR_INVALID, "maxInter missing");
    CK(cudaMemcpyAsync(base + (size_t)P_MAXINTER * N, p->maxInter, 12 * N * sizeof(double),
                       cudaMemcpyHostToDevice, ctx->stream),
       "maxInter");
    if (ctx->proc_pet == -1 || ctx->proc_pet >= 2) { // the same planes hold the PET case's monthly field
        const double *monthly = ctx->proc_pet == -1 ? p->petLAIcorFactor
                                : ctx->proc_pet == 2 ? p->PrieTayAlpha
                                                     : p->aeroResist;
        if (!monthly) return fail(ctx, MHM_ERR_INVALID, "monthly PET parameter (petLAIcorFactor / PrieTayAlpha / "
                                                        "aeroResist) missing");
        CK(cudaMemcpyAsync(base + (size_t)P_PETLAI * N, monthly, 12 * N * sizeof(double), cudaMemcpyHostToDevice,
                           ctx->stream),
           "petLAI");
    }
    if (ctx->proc_pet == 3) {
        if (!p->surfResist) return fail(ctx, MHM_ERR_INVALID, "surfResist missing");
        CK(cudaMemcpyAsync(base + (size_t)P_PET2 * N, p->surfResist, 12 * N * sizeof(double),
                           cudaMemcpyHostToDevice, ctx->stream),
           "surfResist");
    }
    const double *hz[5] = {p->fRoots, p->soilMoistSat, p->soilMoistFC, p->wiltingPoint, p->soilMoistExp};
    for (int g = 0; g < 5; ++g) {
        if (!hz[g]) return fail(ctx, MHM_ERR_INVALID, "horizon parameter missing");
        CK(cudaMemcpyAsync(base + (size_t)(P_HORIZON + g * H) * N, hz[g], (size_t)H * N * sizeof(double),
                           cudaMemcpyHostToDevice, ctx->stream),
           "horizon params");
    }
    CK(cudaStreamSynchronize(ctx->stream), "params sync");
    return MHM_OK;
}

int mhm_set_link_celerity(mhm_ctx *ctx, int32_t m, const double *celerity)
{
    if (!ctx || !celerity) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (ctx->proc_rout != 3) return fail(ctx, MHM_ERR_INVALID, "per-link celerity is routing case 3");
    if (m < 0 || m >= ctx->M) return fail(ctx, MHM_ERR_INVALID, "member out of range");
    if (int rc = mhm_sync(ctx)) return rc; // no enqueued step may still read what changes
    return set_adaptive_member(ctx, m, 0.0, celerity);
}

int mhm_set_meteo_weights(mhm_ctx *ctx, const double *pre_w, const double *pet_w, const double *temp_w)
{
    if (!ctx) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc; // no enqueued step may still read the old weights
    if (!pre_w && !pet_w && !temp_w) {
        ctx->meteo_w_on = false;
        return MHM_OK;
    }
    if (!pre_w || !pet_w || !temp_w)
        return fail(ctx, MHM_ERR_INVALID, "meteo weights come as pre, pet and temp together");
    const size_t n = (size_t)24 * 12 * ctx->N;
    CK(ctx->meteo_w.ensure(3 * n), "meteo weights");
    const double *src[3] = {pre_w, pet_w, temp_w};
    for (int i = 0; i < 3; ++i)
        CK(cudaMemcpyAsync(ctx->meteo_w.p + i * n, src[i], n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream),
           "meteo weights");
    CK(cudaStreamSynchronize(ctx->stream), "meteo weights sync");
    ctx->meteo_w_on = true;
    return MHM_OK;
}

int mhm_set_inflow_gauges(mhm_ctx *ctx, int32_t n, const int32_t *node, const int32_t *headwater)
{
    if (!ctx || n < 0 || (n > 0 && (!node || !headwater))) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc; // no enqueued step may still read the old flags
    if (ctx->proc_rout < 1) return fail(ctx, MHM_ERR_INVALID, "routing is off");
    if (n > kMaxInflow) return fail(ctx, MHM_ERR_UNSUPPORTED, "more than 64 inflow gauges");
    std::vector<int32_t> pos(n);
    std::vector<int8_t> hw(n);
    std::vector<char> cut_node(ctx->L, 0);
    for (int g = 0; g < n; ++g) {
        if (node[g] < 1 || node[g] > ctx->L) return fail(ctx, MHM_ERR_INVALID, "inflow gauge node out of range");
        pos[g] = ctx->net.pos_of_node[node[g] - 1];
        hw[g] = headwater[g] ? 1 : 0;
        if (!hw[g]) cut_node[node[g] - 1] = 1;
    }
    // links draining into a non-headwater gauge's node lose their routed outflow
    std::vector<int8_t> flags = ctx->net.pos_flags;
    for (int i = 0; i < ctx->n_links; ++i)
        if (cut_node[ctx->link_to[i]]) flags[ctx->net.link_pos[i]] |= 4;
    CK(upload(ctx->pos_flags, flags.data(), flags.size(), ctx->stream), "flags");
    if (n > 0) {
        CK(upload(ctx->inflow_pos_d, pos.data(), pos.size(), ctx->stream), "inflow gauges");
        CK(upload(ctx->inflow_hw_d, hw.data(), hw.size(), ctx->stream), "inflow gauges");
    }
    CK(cudaStreamSynchronize(ctx->stream), "inflow sync");
    ctx->n_inflow = n;
    ctx->inflow_pos = pos;
    ctx->inflow_hw = hw;
    return MHM_OK;
}

int mhm_set_inflow_discharge(mhm_ctx *ctx, int32_t day0, int32_t n_days, const double *q)
{
    if (!ctx || n_days < 0 || (n_days > 0 && !q)) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc;
    if (ctx->n_inflow < 1) return fail(ctx, MHM_ERR_INVALID, "no inflow gauges: mhm_set_inflow_gauges first");
    if (day0 < 1) return fail(ctx, MHM_ERR_INVALID, "day0 >= 1 required");
    CK(upload(ctx->inflow_q, q, (size_t)n_days * ctx->n_inflow, ctx->stream), "inflow discharge");
    CK(cudaStreamSynchronize(ctx->stream), "inflow sync");
    ctx->inflow_day0 = day0;
    ctx->inflow_ndays = n_days;
    return MHM_OK;
}

// Where mpr() puts the LAI-indexed parameters: the monthly planes (12 LAI
// entries), or the context's gridded LAI series (as many gridded entries as
// the series has).  Sets a.n_lai_steps / a.lai_out for members member0.. .
static int mpr_lai_target(mhm_ctx *ctx, const MprSetup &m, int32_t member0, MprArgs &a)
{
    a.n_lai_steps = m.n_lai_steps;
    a.lai_out = nullptr;
    if (ctx->lai_mode < 0) {
        if (m.n_lai_classes > 0 || m.n_lai_steps != ctx->n_lai)
            return fail(ctx, MHM_ERR_INVALID, "a gridded LAI series of " + std::to_string(ctx->n_lai) +
                                                  " entries needs gridded L0 LAI with as many entries");
        a.lai_out = ctx->lai_series.p + (size_t)member0 * lai_groups(ctx->proc_pet) * ctx->n_lai * ctx->N;
    } else if (m.n_lai_steps != 12) {
        return fail(ctx, MHM_ERR_INVALID, "L0 LAI with " + std::to_string(m.n_lai_steps) +
                                              " entries needs a gridded LAI series (mhm_set_lai_series)");
    }
    return MHM_OK;
}

int mhm_set_lai_series(mhm_ctx *ctx, int32_t mode, int32_t n_lai)
{
    if (!ctx) return MHM_ERR_INVALID;
    if (mode < -3 || mode > 1) return fail(ctx, MHM_ERR_INVALID, "timeStep_LAI_input must be 1, 0, -1, -2 or -3");
    if (mode < 0 && (n_lai < 1 || n_lai > INT16_MAX))
        return fail(ctx, MHM_ERR_INVALID, "a gridded LAI series needs 1 .. 32767 entries");
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc; // no enqueued step may still read the old series
    if (mode >= 0) {
        ctx->lai_series.release();
        ctx->lai_mode = 0;
        ctx->n_lai = 0;
    } else {
        const size_t n = (size_t)ctx->M * lai_groups(ctx->proc_pet) * n_lai * ctx->N;
        ctx->lai_series.release();
        CK(ctx->lai_series.ensure(n), "LAI series");
        CK(cudaMemsetAsync(ctx->lai_series.p, 0, n * sizeof(double), ctx->stream), "LAI series");
        CK(cudaStreamSynchronize(ctx->stream), "LAI series");
        ctx->lai_mode = mode;
        ctx->n_lai = n_lai;
    }
    ctx->steps_all_filled = 0; // the member step table carries the LAI index
    return MHM_OK;
}

int mhm_set_lai_params(mhm_ctx *ctx, int32_t member, const double *max_inter, const double *pet_lai,
                       const double *surf_resist)
{
    if (!ctx) return MHM_ERR_INVALID;
    if (ctx->lai_mode >= 0) return fail(ctx, MHM_ERR_INVALID, "no gridded LAI series: mhm_set_lai_series first");
    if (member < 0 || member >= ctx->M) return fail(ctx, MHM_ERR_INVALID, "member out of range");
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc;
    const size_t NL = (size_t)ctx->n_lai * ctx->N;
    const int ng = lai_groups(ctx->proc_pet);
    const double *src[3] = {max_inter, pet_lai, surf_resist};
    for (int g = 0; g < ng; ++g) {
        double *dst = ctx->lai_series.p + ((size_t)member * ng + g) * NL;
        if (src[g])
            CK(cudaMemcpyAsync(dst, src[g], NL * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "LAI params");
        else
            CK(cudaMemsetAsync(dst, 0, NL * sizeof(double), ctx->stream), "LAI params");
    }
    CK(cudaStreamSynchronize(ctx->stream), "LAI params");
    return MHM_OK;
}

int mhm_get_lai_params(mhm_ctx *ctx, int32_t member, double *max_inter, double *pet_lai, double *surf_resist)
{
    if (!ctx) return MHM_ERR_INVALID;
    if (ctx->lai_mode >= 0) return fail(ctx, MHM_ERR_INVALID, "no gridded LAI series");
    if (member < 0 || member >= ctx->M) return fail(ctx, MHM_ERR_INVALID, "member out of range");
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc;
    const size_t NL = (size_t)ctx->n_lai * ctx->N;
    double *dst[3] = {max_inter, pet_lai, surf_resist};
    const int ng = lai_groups(ctx->proc_pet);
    for (int g = 0; g < 3; ++g)
        if (dst[g] && g >= ng)
            std::memset(dst[g], 0, NL * sizeof(double)); // a group this PET case does not read
        else if (dst[g])
            CK(cudaMemcpy(dst[g], ctx->lai_series.p + ((size_t)member * ng + g) * NL, NL * sizeof(double),
                          cudaMemcpyDeviceToHost),
               "LAI params");
    return MHM_OK;
}

int mhm_set_link_fpimp(mhm_ctx *ctx, const double *ffp_imp)
{
    if (!ctx || !ffp_imp) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc; // no enqueued step may still use the old fractions
    if (ctx->n_links == 0) return MHM_OK;
    CK(cudaMemcpyAsync(ctx->ffp.p, ffp_imp, (size_t)ctx->n_links * sizeof(double), cudaMemcpyHostToDevice,
                       ctx->stream),
       "fpimp");
    CK(cudaStreamSynchronize(ctx->stream), "fpimp sync");
    return MHM_OK;
}

int mhm_get_eff_params(mhm_ctx *ctx, int32_t m, const mhm_eff_params *p)
{
    if (!ctx || !p) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc;
    if (m < 0 || m >= ctx->M) return fail(ctx, MHM_ERR_INVALID, "member out of range");
    const size_t N = ctx->N;
    const int H = ctx->H, np = n_param_planes(H);
    const double *base = ctx->params.p + (size_t)m * np * N;
    const double *scalars[16] = {p->fSealed,   p->alpha,     p->degDayInc, p->degDayMax,   p->degDayNoPre,
                                 p->fAsp,      p->HarSamCoeff, p->karstLoss, p->kFastFlow, p->kSlowFlow,
                                 p->kBaseFlow, p->kPerco,    p->jarvis_thresh_c1, p->tempThresh, p->unsatThresh,
                                 p->sealedThresh};
    struct Part {
        const double *dst;
        int plane, n_planes;
    };
    const Part parts[] = {{p->maxInter, P_MAXINTER, 12},
                          {ctx->proc_pet >= 2 ? nullptr : p->petLAIcorFactor, P_PETLAI, 12},
                          {ctx->proc_pet == 2 ? p->PrieTayAlpha : nullptr, P_PETLAI, 12},
                          {ctx->proc_pet == 3 ? p->aeroResist : nullptr, P_PETLAI, 12},
                          {ctx->proc_pet == 3 ? p->surfResist : nullptr, P_PET2, 12},
                          {p->fRoots, P_HORIZON, H},              {p->soilMoistSat, P_HORIZON + H, H},
                          {p->soilMoistFC, P_HORIZON + 2 * H, H}, {p->wiltingPoint, P_HORIZON + 3 * H, H},
                          {p->soilMoistExp, P_HORIZON + 4 * H, H}};
    for (int i = 0; i < 16; ++i)
        if (scalars[i])
            CK(cudaMemcpyAsync(const_cast<double *>(scalars[i]), base + (size_t)i * N, N * sizeof(double),
                               cudaMemcpyDeviceToHost, ctx->stream),
               "params");
    for (const Part &q : parts)
        if (q.dst)
            CK(cudaMemcpyAsync(const_cast<double *>(q.dst), base + (size_t)q.plane * N,
                               (size_t)q.n_planes * N * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream),
               "params");
    CK(cudaStreamSynchronize(ctx->stream), "params sync");
    return MHM_OK;
}

int mhm_set_routing_params(mhm_ctx *ctx, int32_t m, const double *p5)
{
    if (!ctx || !p5) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc; // no enqueued step may still read what changes
    if (m < 0 || m >= ctx->M) return fail(ctx, MHM_ERR_INVALID, "member out of range");
    if (ctx->proc_rout == 2) return set_adaptive_member(ctx, m, p5[0], nullptr); // p5[0]: celerity [m s-1]
    if (ctx->proc_rout == 3)
        return fail(ctx, MHM_ERR_INVALID, "routing case 3 takes the links' celerity: mhm_set_link_celerity");
    if (ctx->proc_rout != 1) return fail(ctx, MHM_ERR_INVALID, "routing is off");
    if (ctx->n_links == 0) return MHM_OK;
    const size_t L = ctx->L;
    CK(cudaMemcpyAsync(ctx->rout_p5.p + 5 * m, p5, 5 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream), "p5");
    Bracket br(ctx, 2, ctx->stream);
    CK(launch_reg_rout(ctx->n_links, ctx->rout_p5.p + 5 * m, ctx->ss_max, (double)ctx->timestep, ctx->length.p,
                       ctx->slope.p, ctx->ffp.p, ctx->link_pos.p, ctx->C1.p + m * L, ctx->C2.p + m * L,
                       ctx->stream),
       "reg_rout");
    br.done();
    g_launches++;
    CK(cudaStreamSynchronize(ctx->stream), "reg_rout sync");
    return MHM_OK;
}

int mhm_init_states(mhm_ctx *ctx, int32_t m, const double *hd)
{
    if (!ctx || !hd) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc; // no enqueued step may still read what changes
    if (m < 0 || m >= ctx->M) return fail(ctx, MHM_ERR_INVALID, "member out of range");
    const size_t N = ctx->N;
    const int H = ctx->H, ns = n_state_planes(H);
    // mo_init_states.f90:258-345: interc 0, snow 15, sealed 0, unsat 10, sat 75,
    // SM(h) = (depth(h) - depth(h-1)) * 0.25, last horizon to 1500 mm
    std::vector<double> s((size_t)ns * N);
    auto plane = [&](int pl, double v) { std::fill(s.begin() + (size_t)pl * N, s.begin() + (size_t)(pl + 1) * N, v); };
    plane(S_INTERC, 0.0);
    plane(S_SNOW, 15.0);
    plane(S_SEAL, 0.0);
    plane(S_UNSAT, 10.0);
    plane(S_SAT, 75.0);
    for (int h = 0; h < H - 1; ++h) plane(S_SM + h, (h == 0 ? hd[0] : hd[h] - hd[h - 1]) * 0.25);
    plane(S_SM + H - 1, (1500.0 - (H >= 2 ? hd[H - 2] : 0.0)) * 0.25);
    CK(cudaMemcpyAsync(ctx->states.p + (size_t)m * ns * N, s.data(), s.size() * sizeof(double),
                       cudaMemcpyHostToDevice, ctx->stream),
       "states");
    if (ctx->proc_rout >= 1) {
        const size_t L = ctx->L;
        for (auto *b : {&ctx->qtin1, &ctx->qtr1, &ctx->qout_last, &ctx->qmod_last})
            CK(cudaMemsetAsync(b->p + m * L, 0, L * sizeof(double), ctx->stream), "routing states");
    }
    CK(cudaStreamSynchronize(ctx->stream), "states sync");
    return MHM_OK;
}

int mhm_set_forcing(mhm_ctx *ctx, int32_t kind, int32_t row0, int32_t n_rows, const double *data, int32_t on_device)
{
    if (!ctx) return MHM_ERR_INVALID;
    if (kind < 0 || kind >= kForcKinds) return fail(ctx, MHM_ERR_INVALID, "forcing kind");
    if (row0 < 1 || n_rows < 1 || !data) return fail(ctx, MHM_ERR_INVALID, "forcing rows");
    ForcingSrc &f = ctx->forc[kind];
    f.ptr = data;
    f.row0 = row0;
    f.n_rows = n_rows;
    f.on_device = on_device ? 1 : 0;
    f.set = true;
    return MHM_OK;
}

int mhm_enable_outputs(mhm_ctx *ctx, int32_t total_runoff, int32_t qmod)
{
    if (!ctx) return MHM_ERR_INVALID;
    ctx->out_tro = total_runoff ? 1 : 0;
    ctx->out_qmod = qmod ? 1 : 0;
    return MHM_OK;
}

int mhm_get_outputs(mhm_ctx *ctx, double *total_runoff, double *qmod)
{
    if (!ctx) return MHM_ERR_INVALID;
    if (total_runoff) {
        if (!ctx->out_tro) return fail(ctx, MHM_ERR_INVALID, "total_runoff output not enabled");
        std::memcpy(total_runoff, ctx->host_tro.data(), ctx->host_tro.size() * sizeof(double));
    }
    if (qmod) {
        if (!ctx->out_qmod) return fail(ctx, MHM_ERR_INVALID, "qmod output not enabled");
        std::memcpy(qmod, ctx->host_qmod.data(), ctx->host_qmod.size() * sizeof(double));
    }
    return MHM_OK;
}

// Enqueue n_steps time steps.  Pipeline: the cell chain of every chunk runs
// on `stream`, the L1->L11 accumulation, routing and gauge extraction of the
// same chunk on `route_stream`, so routing of chunk c overlaps the cell chain
// of chunk c+1 (also across calls).  Double-buffered runoff and forcing
// staging slots are guarded by events indexed by a per-context chunk counter.
// hand a staged gauge series to the caller's buffer once its copy is done
static int finish_gauge_stage(mhm_ctx *ctx, mhm_ctx::GaugeStage &st)
{
    if (!st.active) return MHM_OK;
    CK(cudaEventSynchronize(st.ev), "gauge copy");
    std::memcpy(st.dst, st.pinned, st.bytes);
    st.active = false;
    return MHM_OK;
}

// A context's part in a fused multi-context launch of the cell chain
// (mhm_batch_run_members): phase 1 runs run_enqueue up to the cell chain of
// the call's single chunk and returns its launch description; phase 2 runs
// the whole call with the cell chain replaced by a wait for the fused launch.
struct FusedStage {
    int phase = 0;
    CellArgs args{};
    cudaEvent_t ev_fused = nullptr;
};

static int run_enqueue(mhm_ctx *ctx, int32_t tt0, int32_t n_steps, double *q_gauge,
                       const int32_t *member_tt0 = nullptr, FusedStage *fs = nullptr)
{
    NvtxRange nvtx_("mhm: enqueue run");
    if (tt0 < 1 || n_steps < 1) return fail(ctx, MHM_ERR_INVALID, "tt0 >= 1 and n_steps >= 1 required");
    const size_t N = ctx->N, M = ctx->M, L = ctx->L;
    const int H = ctx->H;
    const bool need[kForcKinds] = {true,
                                   true,
                                   ctx->proc_pet == 0 || ctx->proc_pet == -1,
                                   ctx->proc_pet == 1,
                                   ctx->proc_pet == 1,
                                   ctx->proc_pet == 2 || ctx->proc_pet == 3,
                                   ctx->proc_pet == 3,
                                   ctx->proc_pet == 3};
    const int32_t stride = (int32_t)std::lround(24.0 / (double)ctx->ntfd);
    const bool members = member_tt0 != nullptr;
    if (members && (stride != 1 || ctx->ntfd != 24))
        return fail(ctx, MHM_ERR_UNSUPPORTED, "per-member steps need hourly steps with hourly forcing");
    if (members && (ctx->fso.on || ctx->qro.on))
        return fail(ctx, MHM_ERR_UNSUPPORTED, "aggregated outputs with per-member steps");
    for (OutSet *o : {&ctx->fso, &ctx->qro}) {
        if (!o->on) continue;
        const int32_t w = out_advance(*o, ctx->jul_start, ctx->timestep, tt0, n_steps, false);
        if (o->slots + w > o->max_slots)
            return fail(ctx, MHM_ERR_INVALID, "output intervals would exceed the device slots: read the outputs first");
    }
    if (ctx->n_inflow > 0 && ctx->proc_rout >= 1) {
        // the run's days (iDischargeTS) must lie in the inflow discharge series
        const int32_t sd = 24 / ctx->timestep;
        int64_t lo = tt0, hi = (int64_t)tt0 + n_steps - 1;
        if (members) {
            lo = INT64_MAX;
            hi = 0;
            for (size_t m = 0; m < M; ++m)
                if (member_tt0[m] > 0) {
                    lo = std::min<int64_t>(lo, member_tt0[m]);
                    hi = std::max<int64_t>(hi, (int64_t)member_tt0[m] + n_steps - 1);
                }
        }
        if (lo <= hi && ((lo + sd - 1) / sd < ctx->inflow_day0 ||
                         (hi + sd - 1) / sd > (int64_t)ctx->inflow_day0 + ctx->inflow_ndays - 1))
            return fail(ctx, MHM_ERR_INVALID, "inflow discharge does not cover the days of the run");
    }
    if (ctx->lai_mode < 0) {
        // the run's last step must lie in the gridded LAI series (iLAI grows with tt)
        int64_t hi = (int64_t)tt0 + n_steps - 1;
        if (members) {
            hi = 0;
            for (size_t m = 0; m < M; ++m)
                if (member_tt0[m] > 0) hi = std::max<int64_t>(hi, (int64_t)member_tt0[m] + n_steps - 1);
        }
        if (hi >= 1 && step_lai(ctx->jul_start, ctx->timestep, hi, ctx->lai_mode) > ctx->n_lai)
            return fail(ctx, MHM_ERR_INVALID, "the gridded LAI series does not cover the run");
    }
    // member mode reads the first n_steps rows of the device forcing window
    const int32_t first_row = members ? ctx->forc[0].row0 : (tt0 + stride - 1) / stride;
    const int32_t last_row = members ? ctx->forc[0].row0 + n_steps - 1 : (tt0 + n_steps - 1 + stride - 1) / stride;
    int on_device = -1;
    int32_t row0_all = 0;
    for (int k = 0; k < kForcKinds; ++k) {
        if (!need[k]) continue;
        const ForcingSrc &f = ctx->forc[k];
        if (!f.set) return fail(ctx, MHM_ERR_INVALID, "forcing kind " + std::to_string(k) + " not set");
        if (first_row < f.row0 || last_row > f.row0 + f.n_rows - 1)
            return fail(ctx, MHM_ERR_INVALID, "forcing rows do not cover the requested steps");
        if (on_device < 0) {
            on_device = f.on_device;
            row0_all = f.row0;
        }
        if (on_device != f.on_device) return fail(ctx, MHM_ERR_INVALID, "mixed host/device forcing");
        if (on_device && f.row0 != row0_all)
            return fail(ctx, MHM_ERR_INVALID, "device forcing kinds must share row0");
    }
    // chunk length from the total-runoff budget (two slots)
    const size_t per_step = M * N * sizeof(double);
    int32_t Tc = (int32_t)std::max<size_t>(1, std::min<size_t>((size_t)n_steps, ctx->chunk_bytes / (2 * per_step)));
    if (ctx->chunk_cap > 0) Tc = std::min(Tc, ctx->chunk_cap);
    if (!on_device) Tc = std::max<int32_t>(stride, Tc / stride * stride); // whole forcing rows per chunk
    // routing case 2: routing time step shorter than the model step -> R routing
    // passes per step; longer -> one pass per window of F steps
    int32_t R = 1, F = 1;
    if (ctx->proc_rout >= 2 && ctx->L > 1) {
        const double ts = ctx->ts_rout[0];
        for (size_t m = 1; m < M; ++m)
            if (ctx->ts_rout[m] != ts)
                return fail(ctx, MHM_ERR_UNSUPPORTED, "members with different routing time steps");
        if (!(ts > 0.0)) return fail(ctx, MHM_ERR_INVALID, "routing parameters not set");
        const double f = ts / ((double)ctx->timestep * 3600.0);
        if (f < 1.0)
            R = std::max<int32_t>(1, (int32_t)std::lround(1.0 / f));
        else
            F = std::max<int32_t>(1, (int32_t)std::lround(f));
        if (F > 1) {
            if (members) return fail(ctx, MHM_ERR_UNSUPPORTED, "per-member steps with a multi-step routing window");
            if ((tt0 - 1) % F != 0 || n_steps % F != 0)
                return fail(ctx, MHM_ERR_INVALID,
                            "runs must cover whole routing steps of " + std::to_string(F) + " model steps");
            Tc = std::max<int32_t>(F, Tc / F * F);
        }
    }
    if (ctx->tc_cap < Tc) {
        // growing the per-chunk buffers: no older work may still use them
        CK(cudaStreamSynchronize(ctx->stream), "sync");
        CK(cudaStreamSynchronize(ctx->route_stream), "sync");
        CK(cudaStreamSynchronize(ctx->copy_stream), "sync");
        for (int s = 0; s < 2; ++s) CK(ctx->tro[s].ensure((size_t)Tc * M * N), "total runoff chunk");
        if (ctx->proc_rout >= 1) {
            CK(ctx->qout.ensure(M * (size_t)Tc * L), "qout chunk");
            CK(ctx->qtr.ensure(M * (size_t)Tc * L), "qtr chunk");
            CK(ctx->qmod.ensure(M * (size_t)Tc * L), "qmod chunk");
        }
        const int32_t max_rows = (Tc + stride - 1) / stride + 1;
        for (int k = 0; k < kForcKinds; ++k)
            for (int s = 0; s < 2; ++s) ctx->stage[k][s].release();
        ctx->stage_rows = max_rows;
        ctx->tc_cap = Tc;
    }
    if ((R > 1 || F > 1) && ctx->proc_rout >= 1) {
        const size_t need_rt = M * (size_t)ctx->tc_cap * R * L;
        if (ctx->qtr.n < need_rt || ctx->qmod_sub.n < need_rt) {
            CK(cudaStreamSynchronize(ctx->route_stream), "sync");
            CK(ctx->qtr.ensure(need_rt), "qtr routing steps");
            CK(ctx->qmod_sub.ensure(need_rt), "qmod routing steps");
        }
    }
    if (!on_device)
        for (int k = 0; k < kForcKinds; ++k)
            if (need[k])
                for (int s = 0; s < 2; ++s) CK(ctx->stage[k][s].ensure((size_t)ctx->stage_rows * N), "forcing staging");
    if (ctx->proc_rout >= 1 && ctx->G > 0 && q_gauge) {
        // one device gauge buffer per call in flight: ring of 2
        const int gs = (int)(ctx->call_seq & 1);
        if (ctx->qg_cap[gs] < M * (size_t)ctx->G * n_steps) {
            CK(cudaStreamSynchronize(ctx->route_stream), "sync");
            CK(ctx->q_gauge[gs].ensure(M * (size_t)ctx->G * n_steps), "q_gauge");
            ctx->qg_cap[gs] = M * (size_t)ctx->G * n_steps;
        }
    }
    if (ctx->out_tro) ctx->host_tro.assign((size_t)n_steps * M * N, 0.0);
    if (ctx->out_flux) {
        for (int k = 0; k < 2; ++k) CK(ctx->flux_d[k].ensure((size_t)ctx->tc_cap * M * N), "flux outputs");
        ctx->host_aet.assign((size_t)n_steps * M * N, 0.0);
        ctx->host_loss.assign((size_t)n_steps * M * N, 0.0);
    }
    if (ctx->out_qmod) ctx->host_qmod.assign(M * (size_t)n_steps * L, 0.0);
    const int nchunks = (n_steps + Tc - 1) / Tc;
    if (fs && (nchunks != 1 || !members))
        return fail(ctx, MHM_ERR_UNSUPPORTED, "a fused launch takes one chunk of per-member steps per context ("
                                              "n_steps " + std::to_string(n_steps) + " > chunk " + std::to_string(Tc) + ")");
    auto chunk_rows = [&](int c, int32_t &r0, int32_t &r1) { // forcing rows iMeteoTS of the chunk
        const int64_t t0 = (int64_t)tt0 + c * Tc, t1 = (int64_t)tt0 + std::min(n_steps, (c + 1) * Tc) - 1;
        r0 = (int32_t)((t0 + stride - 1) / stride);
        r1 = (int32_t)((t1 + stride - 1) / stride);
    };
    const int64_t seq0 = ctx->chunk_seq;
    auto issue_copy = [&](int c) -> int {
        if (on_device || c >= nchunks) return MHM_OK;
        const int slot = (int)((seq0 + c) & 1);
        int32_t r0, r1;
        chunk_rows(c, r0, r1);
        if (ctx->slot_used[slot]) CK(cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_consumed[slot], 0), "wait slot");
        for (int k = 0; k < kForcKinds; ++k) {
            if (!need[k]) continue;
            const ForcingSrc &f = ctx->forc[k];
            CK(cudaMemcpyAsync(ctx->stage[k][slot].p, f.ptr + (size_t)(r0 - f.row0) * N,
                               (size_t)(r1 - r0 + 1) * N * sizeof(double), cudaMemcpyHostToDevice, ctx->copy_stream),
               "forcing H2D");
        }
        CK(cudaEventRecord(ctx->ev_copied[slot], ctx->copy_stream), "record copied");
        return MHM_OK;
    };
    if (members) {
        if (!on_device) return fail(ctx, MHM_ERR_INVALID, "per-member steps need device forcing");
        int32_t max_t0 = 0;
        ctx->member_s0_h.assign(M, -1);
        for (size_t m = 0; m < M; ++m) {
            if (member_tt0[m] > 0) ctx->member_s0_h[m] = member_tt0[m] - 1;
            max_t0 = std::max(max_t0, member_tt0[m]);
        }
        const int64_t need_steps = (int64_t)std::max(max_t0, 1) - 1 + n_steps;
        if (need_steps > ctx->steps_all_filled) {
            // calendar of steps 1 .. need_steps (grown in 8760-step blocks)
            const int64_t cap = ((need_steps + 8759) / 8760) * 8760;
            CK(cudaStreamSynchronize(ctx->stream), "sync");
            CK(ctx->steps_all.ensure((size_t)cap), "member steps");
            CK(launch_steps_fill(ctx->steps_all.p, 1, (int32_t)cap, ctx->jul_start, ctx->timestep, 1, ctx->lai_mode,
                                 ctx->stream),
               "steps fill");
            g_launches++;
            ctx->steps_all_filled = cap;
        }
        if (!(fs && fs->phase == 2)) { // phase 2 reuses the table phase 1 uploaded
            const int r = (int)(ctx->member_calls & 3);
            if (!ctx->ev_members_done[r]) {
                CK(cudaEventCreateWithFlags(&ctx->ev_members_done[r], cudaEventDisableTiming), "event");
            } else {
                CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_members_done[r], 0), "wait member table");
            }
            CK(ctx->member_s0[r].ensure(M), "member steps");
            CK(cudaMemcpyAsync(ctx->member_s0[r].p, ctx->member_s0_h.data(), M * sizeof(int32_t),
                               cudaMemcpyHostToDevice, ctx->stream),
               "member steps");
            ctx->member_s0_cur = ctx->member_s0[r].p;
        }
    }
    if (ctx->timing && !ctx->run_a) {
        cudaEventCreate(&ctx->run_a);
        cudaEventRecord(ctx->run_a, ctx->stream);
    }
    if (int rc = issue_copy(0)) return rc;
    for (int c = 0; c < nchunks; ++c) {
        if (int rc = issue_copy(c + 1)) return rc;
        const int32_t s0 = c * Tc;
        const int32_t nT = std::min(n_steps, s0 + Tc) - s0;
        const int slot = (int)((seq0 + c) & 1);
        // this chunk's calendar, computed on the device (stream-ordered before the cell chain)
        if (!members) {
            CK(ctx->steps.ensure((size_t)ctx->tc_cap), "steps");
            CK(launch_steps_fill(ctx->steps.p, tt0 + s0, nT, ctx->jul_start, ctx->timestep, stride, ctx->lai_mode,
                                 ctx->stream),
               "steps fill");
            g_launches++;
        }
        // the runoff slot must have been consumed by the accumulation of chunk (seq - 2)
        if (ctx->slot_used[slot]) CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_acc_done[slot], 0), "wait acc");
        CellArgs a{};
        a.n_cells = ctx->N;
        a.n_members = ctx->M;
        a.n_steps = nT;
        a.proc_sm = ctx->proc_sm;
        a.proc_pet = ctx->proc_pet;
        a.is_hourly = ctx->ntfd == 24;
        a.reset_sm = (tt0 + s0 == 1) && !ctx->read_states;
        a.c2TSTu = (double)ctx->timestep / 24.0;
        a.nTstepDay = 24.0 / (double)ctx->timestep;
        const double *fp[kForcKinds] = {};
        if (on_device) {
            a.row_base = row0_all;
            a.n_forc_rows = INT32_MAX;
            for (int k = 0; k < kForcKinds; ++k)
                if (need[k]) {
                    fp[k] = ctx->forc[k].ptr;
                    a.n_forc_rows = std::min(a.n_forc_rows, ctx->forc[k].n_rows);
                }
        } else {
            int32_t r0, r1;
            chunk_rows(c, r0, r1);
            a.row_base = r0;
            a.n_forc_rows = r1 - r0 + 1;
            for (int k = 0; k < kForcKinds; ++k)
                if (need[k]) fp[k] = ctx->stage[k][slot].p;
            CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_copied[slot], 0), "wait copied");
        }
        a.pre = fp[0];
        a.temp = fp[1];
        a.pet = fp[2];
        a.tmin = fp[3];
        a.tmax = fp[4];
        a.netrad = fp[5];
        a.eabs = fp[6];
        a.wind = fp[7];
        if (ctx->meteo_w_on) {
            const size_t wn = (size_t)24 * 12 * N;
            a.w_pre = ctx->meteo_w.p;
            a.w_pet = ctx->meteo_w.p + wn;
            a.w_temp = ctx->meteo_w.p + 2 * wn;
        }
        a.steps = ctx->steps.p;
        if (members) {
            a.steps = ctx->steps_all.p;
            a.n_step_rows = (int32_t)std::min<int64_t>(ctx->steps_all_filled, INT32_MAX);
            a.member_step0 = ctx->member_s0_cur;
            a.step_shift = s0;
            a.reset_ok = !ctx->read_states;
            a.reset_sm = 0;
        }
        a.params = ctx->params.p;
        a.states = ctx->states.p;
        a.tro = ctx->tro[slot].p;
        a.latitude = ctx->latitude.p;
        a.tab = ctx->tab;
        a.nonfinite = ctx->nonfinite.p;
        a.n_horizons = H;
        if (ctx->lai_mode < 0) {
            a.lai_series = ctx->lai_series.p;
            a.n_lai = ctx->n_lai;
        }
        if (ctx->out_flux) {
            a.flux_aet = ctx->flux_d[0].p;
            a.flux_loss = ctx->flux_d[1].p;
        }
        if (ctx->fso.on) {
            OutArgs &o = a.out;
            o.n_planes = ctx->fso.n_planes;
            o.interval = ctx->fso.interval;
            o.warm_steps = ctx->fso.warm;
            o.n_tt = ctx->fso.n_tt;
            o.tt_base = (int64_t)tt0 + s0;
            o.slot0 = ctx->fso.slots;
            o.cnt0 = ctx->fso.cnt;
            o.max_slots = ctx->fso.max_slots;
            std::memcpy(o.plane, ctx->fs_plane, sizeof(o.plane));
            o.avg_mask = ctx->fs_avg;
            o.acc = ctx->fso.acc.p;
            o.out = ctx->fso.out.p;
            o.tt_w = ctx->w_tt.p;
            o.w_fsealed = ctx->w_fs.p;
            o.w_sms = ctx->w_sms.p;
            out_advance(ctx->fso, ctx->jul_start, ctx->timestep, (int64_t)tt0 + s0, nT, true);
        }
        if (fs && fs->phase == 1) {
            fs->args = a; // everything up to the cell chain is enqueued; the rest follows in phase 2
            return MHM_OK;
        }
        if (fs) {
            CK(cudaStreamWaitEvent(ctx->stream, fs->ev_fused, 0), "wait fused cell chain");
        } else {
            Bracket br(ctx, 0, ctx->stream);
            CK(launch_cell_chain(a, H, ctx->cell_occ, ctx->stream), "cell chain launch");
            br.done();
            g_launches++;
        }
        if (ctx->out_tro)
            CK(cudaMemcpyAsync(ctx->host_tro.data() + (size_t)s0 * M * N, ctx->tro[slot].p,
                               (size_t)nT * M * N * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream),
               "tro D2H");
        if (ctx->out_flux) {
            CK(cudaMemcpyAsync(ctx->host_aet.data() + (size_t)s0 * M * N, ctx->flux_d[0].p,
                               (size_t)nT * M * N * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream),
               "flux D2H");
            CK(cudaMemcpyAsync(ctx->host_loss.data() + (size_t)s0 * M * N, ctx->flux_d[1].p,
                               (size_t)nT * M * N * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream),
               "flux D2H");
        }
        if (!on_device) CK(cudaEventRecord(ctx->ev_consumed[slot], ctx->stream), "record consumed");
        CK(cudaEventRecord(ctx->ev_cell_done[slot], ctx->stream), "record cell done");
        ctx->slot_used[slot] = true;
        // ---- routing of this chunk on route_stream ----
        NvtxRange nvtx_route("mhm: routing chunk");
        cudaStream_t rs = ctx->route_stream;
        CK(cudaStreamWaitEvent(rs, ctx->ev_cell_done[slot], 0), "wait cell");
        if (ctx->proc_rout >= 1) {
            AccArgs acc{};
            acc.n_cells = ctx->N;
            acc.n_nodes = ctx->L;
            acc.n_members = ctx->M;
            acc.n_steps = nT / F;
            acc.map_flag = ctx->map_flag;
            acc.win = F;
            acc.TST = 3600.0 * (ctx->timestep * F);
            acc.tro = ctx->tro[slot].p;
            acc.l1_area = ctx->l1_area.p;
            acc.node_cell_ptr = ctx->node_cell_ptr.p;
            acc.node_cells = ctx->node_cells.p;
            acc.pos_l11_l1 = ctx->pos_l11_l1.p;
            acc.pos_area = ctx->pos_area.p;
            acc.qout = ctx->qout.p;
            acc.member_step0 = members ? ctx->member_s0_cur : nullptr;
            {
                Bracket br(ctx, 1, rs);
                CK(launch_runoff_acc(acc, rs), "runoff acc launch");
                br.done();
                g_launches++;
            }
        }
        if (ctx->proc_rout >= 1 && ctx->n_inflow > 0) {
            InflowArgs ia{};
            ia.n_members = ctx->M;
            ia.n_qsteps = nT / F;
            ia.n_nodes = ctx->L;
            ia.n_inflow = ctx->n_inflow;
            ia.win = F;
            ia.steps_day = 24 / ctx->timestep;
            ia.day0 = ctx->inflow_day0;
            // adaptive routing with a routing step not shorter than the model step:
            // the routing step's mean (mo_mhm_interface_run.f90:497-510)
            const double tsf = (ctx->proc_rout >= 2 && ctx->L > 1)
                                   ? ctx->ts_rout[0] / ((double)ctx->timestep * 3600.0) : 1.0;
            ia.mean = (ctx->proc_rout >= 2 && ctx->L > 1 && !(tsf < 1.0)) ? 1 : 0;
            ia.tsf = tsf;
            ia.tt_base = (int64_t)tt0 + s0;
            ia.member_step0 = members ? ctx->member_s0_cur : nullptr;
            ia.step_shift = s0;
            ia.pos = ctx->inflow_pos_d.p;
            ia.headwater = ctx->inflow_hw_d.p;
            ia.q = ctx->inflow_q.p;
            ia.n_days = ctx->inflow_ndays;
            ia.qout = ctx->qout.p;
            CK(launch_inflow(ia, rs), "inflow launch");
            g_launches++;
        }
        CK(cudaEventRecord(ctx->ev_acc_done[slot], rs), "record acc done");
        if (ctx->proc_rout < 1) continue;
        RouteArgs r{};
        const int32_t n_rsteps = nT * R / F; // routing steps of the chunk
        r.n_nodes = ctx->L;
        r.n_members = ctx->M;
        r.n_steps = n_rsteps;
        r.rdiv = R;
        r.n_qsteps = nT / F;
        r.sub = std::min(ctx->route_sub, n_rsteps);
        r.pos_level = ctx->pos_level.p;
        r.up_ptr = ctx->up_ptr.p;
        r.up_pos = ctx->up_pos.p;
        r.pos_flags = ctx->pos_flags.p;
        r.C1 = ctx->C1.p;
        r.C2 = ctx->C2.p;
        r.qout = ctx->qout.p;
        r.qtr = ctx->qtr.p;
        r.qmod = (R > 1 || F > 1) ? ctx->qmod_sub.p : ctx->qmod.p;
        r.qtin1 = ctx->qtin1.p;
        r.qtr1 = ctx->qtr1.p;
        r.member_step0 = members ? ctx->member_s0_cur : nullptr;
        {
            Bracket br(ctx, 2, rs);
            // wavefront: tick k advances sub-chunk k - l of level l
            const int D = ctx->net.n_levels;
            const int n_sub = (n_rsteps + r.sub - 1) / r.sub;
            const int n_ticks = D + n_sub - 1;
            auto enqueue_ticks = [&]() -> int {
                if (ctx->route_cluster > 0) { // all ticks in one launch
                    RouteWalk w{};
                    w.level_ptr = ctx->level_ptr_d.p;
                    w.n_levels = D;
                    w.n_sub = n_sub;
                    w.n_ticks = n_ticks;
                    CK(launch_route_walk(r, w, ctx->route_cluster, rs), "route walk launch");
                    return MHM_OK;
                }
                for (int k = 0; k < n_ticks; ++k) {
                    const int lo = std::max(0, k - n_sub + 1), hi = std::min(k, D - 1);
                    r.tick = k;
                    r.pos_begin = ctx->net.level_ptr[lo];
                    r.pos_end = ctx->net.level_ptr[hi + 1];
                    CK(launch_route_tick(r, rs), "route launch");
                }
                return MHM_OK;
            };
            if (ctx->route_graphs_on && ctx->route_cluster == 0) {
                auto &cache = ctx->route_graphs;
                auto it = std::find_if(cache.begin(), cache.end(),
                                       [&](const RouteGraph &g) { return same_route_shape(g.key, r); });
                if (it == cache.end()) {
                    RouteGraph rg;
                    rg.key = r;
                    rg.n_ticks = n_ticks;
                    cudaGraph_t graph = nullptr;
                    CK(cudaStreamBeginCapture(rs, cudaStreamCaptureModeThreadLocal), "route capture");
                    const int rc_cap = enqueue_ticks();
                    const cudaError_t e_end = cudaStreamEndCapture(rs, &graph);
                    if (rc_cap) {
                        if (graph) cudaGraphDestroy(graph);
                        return rc_cap;
                    }
                    CK(e_end, "route capture end");
                    const cudaError_t e_inst = cudaGraphInstantiate(&rg.exec, graph, 0);
                    cudaGraphDestroy(graph);
                    CK(e_inst, "route graph instantiate");
                    if (cache.size() >= 8) { // keep the most recently used shapes
                        cudaGraphExecDestroy(cache.front().exec);
                        cache.erase(cache.begin());
                    }
                    cache.push_back(rg);
                    it = cache.end() - 1;
                } else if (it != cache.end() - 1) {
                    std::rotate(it, it + 1, cache.end());
                    it = cache.end() - 1;
                }
                CK(cudaGraphLaunch(it->exec, rs), "route graph launch");
            } else if (int rc = enqueue_ticks()) {
                return rc;
            }
            g_launches += ctx->route_cluster > 0 ? 1 : n_ticks;
            if (R > 1 || F > 1) {
                QmodStepArgs qs{};
                qs.n_members = ctx->M;
                qs.n_steps = nT;
                qs.n_nodes = ctx->L;
                qs.rdiv = R;
                qs.win = F;
                qs.qmod_sub = ctx->qmod_sub.p;
                qs.qmod = ctx->qmod.p;
                qs.member_step0 = r.member_step0;
                CK(launch_qmod_step(qs, rs), "qmod step launch");
                g_launches++;
            }
            br.done();
        }
        if (ctx->G > 0 && q_gauge) {
            GaugeArgs g{};
            g.n_members = ctx->M;
            g.n_steps = nT;
            g.n_nodes = ctx->L;
            g.n_gauges = ctx->G;
            g.step_offset = s0;
            g.total_steps = n_steps;
            g.gauge_pos = ctx->gauge_pos_d.p;
            g.qmod = ctx->qmod.p;
            g.q_gauge = ctx->q_gauge[(int)(ctx->call_seq & 1)].p;
            g.member_step0 = members ? ctx->member_s0_cur : nullptr;
            CK(launch_gauge_gather(g, rs), "gauge launch");
            g_launches++;
        }
        if (ctx->out_qmod)
            for (size_t m = 0; m < M; ++m)
                CK(cudaMemcpyAsync(ctx->host_qmod.data() + (m * n_steps + s0) * L, ctx->qmod.p + m * (size_t)nT * L,
                                   (size_t)nT * L * sizeof(double), cudaMemcpyDeviceToHost, rs),
                   "qmod D2H");
        if (ctx->qro.on) {
            QroutArgs qa{};
            qa.n_members = ctx->M;
            qa.n_steps = nT;
            qa.n_nodes = ctx->L;
            qa.win = F;
            qa.interval = ctx->qro.interval;
            qa.slot0 = ctx->qro.slots;
            qa.cnt0 = ctx->qro.cnt;
            qa.max_slots = ctx->qro.max_slots;
            qa.warm_steps = ctx->qro.warm;
            qa.n_tt = ctx->qro.n_tt;
            qa.tt_base = (int64_t)tt0 + s0;
            qa.jul_start = ctx->jul_start;
            qa.timestep = ctx->timestep;
            qa.qmod = ctx->qmod.p;
            qa.qmod_prev = ctx->qmod_last.p;
            qa.acc = ctx->qro.acc.p;
            qa.out = ctx->qro.out.p;
            CK(launch_qrouted(qa, rs), "Qrouted launch");
            g_launches++;
            out_advance(ctx->qro, ctx->jul_start, ctx->timestep, (int64_t)tt0 + s0, nT, true);
        }
        if (c == nchunks - 1 || ctx->qro.on) {
            // qOUT and Qmod of the chunk's last step (restart fields; the
            // Qrouted output of the next chunk starts from this Qmod)
            for (size_t m = 0; m < M; ++m) {
                if (members && ctx->member_s0_h[m] < 0) continue; // idle member keeps its restart fields
                const size_t nq = (size_t)(nT / F); // qOUT rows: one per routing step of the window mode
                CK(cudaMemcpyAsync(ctx->qout_last.p + m * L, ctx->qout.p + (m * nq + (nq - 1)) * L, L * sizeof(double),
                                   cudaMemcpyDeviceToDevice, rs),
                   "qout last");
                CK(cudaMemcpyAsync(ctx->qmod_last.p + m * L, ctx->qmod.p + (m * nT + (nT - 1)) * L, L * sizeof(double),
                                   cudaMemcpyDeviceToDevice, rs),
                   "qmod last");
            }
        }
    }
    ctx->chunk_seq += nchunks;
    if (q_gauge && ctx->proc_rout >= 1 && ctx->G > 0) {
        auto &st = ctx->qg_stage[(int)(ctx->call_seq & 1)];
        const size_t bytes = M * (size_t)ctx->G * n_steps * sizeof(double);
        if (int rc = finish_gauge_stage(ctx, st)) return rc; // the call two back used this slot
        if (st.cap < bytes) {
            if (st.pinned) cudaFreeHost(st.pinned);
            st.pinned = nullptr;
            st.cap = 0;
            CK(cudaMallocHost((void **)&st.pinned, bytes), "gauge staging");
            st.cap = bytes;
        }
        if (!st.ev) CK(cudaEventCreateWithFlags(&st.ev, cudaEventDisableTiming), "event");
        CK(cudaMemcpyAsync(st.pinned, ctx->q_gauge[(int)(ctx->call_seq & 1)].p, bytes, cudaMemcpyDeviceToHost,
                           ctx->route_stream),
           "q_gauge D2H");
        CK(cudaEventRecord(st.ev, ctx->route_stream), "record gauge copy");
        st.dst = q_gauge;
        st.bytes = bytes;
        st.active = true;
    }
    if (members) {
        // the table may be reused once this call's routing has finished
        CK(cudaEventRecord(ctx->ev_members_done[ctx->member_calls & 3], ctx->route_stream), "record member table");
        ctx->member_calls += 1;
    }
    ctx->call_seq += 1;
    ctx->last_steps = n_steps;
    ctx->pending_outputs = ctx->out_tro || ctx->out_qmod;
    return MHM_OK;
}

int mhm_poll(mhm_ctx *ctx, int32_t *done)
{
    if (!ctx || !done) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    // events recorded now cover everything enqueued so far on the streams
    if (!ctx->ev_poll[0])
        for (auto &e : ctx->ev_poll) CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "event");
    cudaStream_t ss[3] = {ctx->stream, ctx->route_stream, ctx->copy_stream};
    *done = 1;
    for (int i = 0; i < 3; ++i) {
        CK(cudaEventRecord(ctx->ev_poll[i], ss[i]), "poll record");
        const cudaError_t e = cudaEventQuery(ctx->ev_poll[i]);
        if (e == cudaErrorNotReady) {
            *done = 0;
        } else if (e != cudaSuccess) {
            return cuda_fail(ctx, e, "poll");
        }
    }
    return MHM_OK;
}

// The bounds-checked build's status for the work that has completed on the
// context's device: MHM_OK, or MHM_ERR_BOUNDS with the site and index of the
// first failed index test (status words read and cleared).
static int take_bounds_status(mhm_ctx *ctx, int32_t *site, int64_t *index)
{
    if (site) *site = 0;
    if (index) *index = 0;
    if (!kBoundsChecked) return MHM_OK;
    cudaError_t (*const readers[])(unsigned long long *) = {bc_take_cell_chain, bc_take_cell_chain_o6,
                                                            bc_take_cell_chain_o8, bc_take_routing, bc_take_mpr};
    unsigned long long first = 0;
    for (auto rd : readers) {
        unsigned long long v = 0;
        CK(rd(&v), "bounds status");
        if (v && !first) first = v;
    }
    if (!first) return MHM_OK;
    const int32_t st = (int32_t)(first >> 48);
    const int64_t ix = (int64_t)(first & 0xffffffffffffULL);
    if (site) *site = st;
    if (index) *index = ix;
    return fail(ctx, MHM_ERR_BOUNDS,
                "index out of range at check site " + std::to_string(st) + " (index " + std::to_string(ix) + ")");
}

int mhm_bounds_checked(void) { return kBoundsChecked ? 1 : 0; }

int mhm_device_status(mhm_ctx *ctx, int32_t *site, int64_t *index)
{
    if (!ctx) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    CK(cudaStreamSynchronize(ctx->stream), "sync");
    CK(cudaStreamSynchronize(ctx->route_stream), "sync");
    CK(cudaStreamSynchronize(ctx->copy_stream), "sync");
    return take_bounds_status(ctx, site, index);
}

int mhm_bounds_selftest(mhm_ctx *ctx)
{
    if (!ctx) return MHM_ERR_INVALID;
    if (!kBoundsChecked) return fail(ctx, MHM_ERR_UNSUPPORTED, "not a bounds-checked build");
    ON_CTX_DEVICE(ctx);
    CK(cudaStreamSynchronize(ctx->stream), "sync");
    CK(launch_bc_selftest(ctx->stream), "self-test launch");
    CK(cudaStreamSynchronize(ctx->stream), "sync");
    return MHM_OK;
}

int mhm_sync(mhm_ctx *ctx)
{
    NvtxRange nvtx_("mhm: sync");
    if (!ctx) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (ctx->timing && ctx->run_a) {
        cudaEvent_t b;
        cudaEventCreate(&b);
        cudaEventRecord(b, ctx->route_stream);
        ctx->pending.push_back({3, ctx->run_a, b});
        ctx->run_a = nullptr;
    }
    // leave `stream` ordered after all routing work
    CK(cudaEventRecord(ctx->ev_route_end, ctx->route_stream), "record route end");
    CK(cudaStreamWaitEvent(ctx->stream, ctx->ev_route_end, 0), "join");
    CK(cudaStreamSynchronize(ctx->stream), "run sync");
    CK(cudaStreamSynchronize(ctx->copy_stream), "copy sync");
    for (auto &st : ctx->qg_stage)
        if (int rc = finish_gauge_stage(ctx, st)) return rc;
    harvest_timing(ctx);
    if (int rc = take_bounds_status(ctx, nullptr, nullptr)) return rc;
    if (ctx->pending_outputs && ctx->out_qmod) { // routing-level positions -> node order
        const size_t L = ctx->L;
        std::vector<double> row(L);
        for (size_t r = 0; r < (size_t)ctx->M * (size_t)ctx->last_steps; ++r) {
            double *q = ctx->host_qmod.data() + r * L;
            for (size_t v = 0; v < L; ++v) row[v] = q[ctx->net.pos_of_node[v]];
            std::memcpy(q, row.data(), L * sizeof(double));
        }
    }
    ctx->pending_outputs = false;
    return MHM_OK;
}

int mhm_run_async(mhm_ctx *ctx, int32_t tt0, int32_t n_steps, double *q_gauge)
{
    if (!ctx) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (ctx->out_tro || ctx->out_qmod || ctx->out_flux)
        return fail(ctx, MHM_ERR_INVALID, "per-step outputs need the synchronous mhm_run");
    return run_enqueue(ctx, tt0, n_steps, q_gauge);
}

int mhm_run_members_async(mhm_ctx *ctx, const int32_t *member_tt0, int32_t n_steps, double *q_gauge)
{
    if (!ctx || !member_tt0) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (ctx->out_tro || ctx->out_qmod || ctx->out_flux)
        return fail(ctx, MHM_ERR_INVALID, "per-step outputs need the synchronous mhm_run");
    return run_enqueue(ctx, 1, n_steps, q_gauge, member_tt0);
}

int mhm_snapshot_alloc(mhm_ctx *ctx, int32_t n_slots)
{
    if (!ctx || n_slots < 0) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc;
    const size_t per = (size_t)n_state_planes(ctx->H) * ctx->N + 4 * (size_t)ctx->L;
    ctx->snap.release();
    ctx->n_snap = 0;
    CK(ctx->snap.ensure(per * (size_t)n_slots), "snapshots");
    ctx->n_snap = n_slots;
    return MHM_OK;
}

// device-to-device copy of one member's states (cells and routing) to or from
// a snapshot slot, ordered after all work enqueued on the context
static int snapshot_copy(mhm_ctx *ctx, int32_t member, int32_t slot, bool save)
{
    if (!ctx) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (member < 0 || member >= ctx->M || slot < 0 || slot >= ctx->n_snap)
        return fail(ctx, MHM_ERR_INVALID, "member or snapshot slot out of range");
    const size_t N = ctx->N, L = ctx->L, ns = n_state_planes(ctx->H);
    const size_t per = ns * N + 4 * L;
    double *sp = ctx->snap.p + (size_t)slot * per;
    struct Part {
        double *member_ptr;
        size_t n;
    };
    const Part parts[5] = {{ctx->states.p + (size_t)member * ns * N, ns * N},
                           {ctx->qtin1.p ? ctx->qtin1.p + (size_t)member * L : nullptr, L},
                           {ctx->qtr1.p ? ctx->qtr1.p + (size_t)member * L : nullptr, L},
                           {ctx->qout_last.p ? ctx->qout_last.p + (size_t)member * L : nullptr, L},
                           {ctx->qmod_last.p ? ctx->qmod_last.p + (size_t)member * L : nullptr, L}};
    cudaStream_t s = ctx->stream;
    CK(cudaEventRecord(ctx->ev_route_end, ctx->route_stream), "record route end");
    CK(cudaStreamWaitEvent(s, ctx->ev_route_end, 0), "join");
    size_t off = 0;
    for (const Part &q : parts) {
        if (q.member_ptr && q.n) {
            double *dst = save ? sp + off : q.member_ptr;
            const double *src = save ? q.member_ptr : sp + off;
            CK(cudaMemcpyAsync(dst, src, q.n * sizeof(double), cudaMemcpyDeviceToDevice, s), "snapshot copy");
        }
        off += q.n;
    }
    return MHM_OK;
}

int mhm_snapshot_save(mhm_ctx *ctx, int32_t member, int32_t slot) { return snapshot_copy(ctx, member, slot, true); }

int mhm_snapshot_load(mhm_ctx *ctx, int32_t slot, int32_t member) { return snapshot_copy(ctx, member, slot, false); }

int mhm_set_launch_config(mhm_ctx *ctx, const mhm_launch_config *cfg)
{
    if (!ctx || !cfg) return MHM_ERR_INVALID;
    if (cfg->cell_blocks_per_sm != 4 && cfg->cell_blocks_per_sm != 6 && cfg->cell_blocks_per_sm != 8)
        return fail(ctx, MHM_ERR_INVALID, "cell_blocks_per_sm must be 4, 6 or 8");
    if (cfg->route_sub_steps < 1 || cfg->route_sub_steps > 16)
        return fail(ctx, MHM_ERR_INVALID, "route_sub_steps must be 1..16");
    if (cfg->chunk_steps < 0) return fail(ctx, MHM_ERR_INVALID, "chunk_steps must be >= 0");
    if (cfg->route_cluster != 0 && cfg->route_cluster != 4 && cfg->route_cluster != 8 && cfg->route_cluster != 16)
        return fail(ctx, MHM_ERR_INVALID, "route_cluster must be 0, 4, 8 or 16");
    if (int rc = mhm_sync(ctx)) return rc;
    ctx->cell_occ = cfg->cell_blocks_per_sm;
    ctx->route_sub = cfg->route_sub_steps;
    ctx->chunk_cap = cfg->chunk_steps;
    ctx->route_cluster = cfg->route_cluster;
    return MHM_OK;
}

int mhm_get_launch_config(mhm_ctx *ctx, mhm_launch_config *cfg)
{
    if (!ctx || !cfg) return MHM_ERR_INVALID;
    cfg->cell_blocks_per_sm = ctx->cell_occ;
    cfg->route_sub_steps = ctx->route_sub;
    cfg->chunk_steps = ctx->chunk_cap;
    cfg->route_cluster = ctx->route_cluster;
    return MHM_OK;
}

// The autotuners' trial runs: every trial starts from the same states (a
// device copy taken first and put back after each trial and at the end), the
// outputs are switched off while trials run, and a trial is timed with events
// from its first enqueue to the join of all streams.
struct TuneScope {
    mhm_ctx *ctx;
    DevBuf<double> keep;
    size_t n_cells_st = 0, n_rt = 0;
    bool rout = false;
    int32_t out_t = 0, out_q = 0, out_f = 0;
    bool fso_on = false, qro_on = false;
    cudaEvent_t e0 = nullptr, e1 = nullptr;

    explicit TuneScope(mhm_ctx *c) : ctx(c)
    {
        out_t = ctx->out_tro;
        out_q = ctx->out_qmod;
        out_f = ctx->out_flux;
        ctx->out_tro = ctx->out_qmod = ctx->out_flux = 0;
        fso_on = ctx->fso.on; // trials add nothing to the outputs
        qro_on = ctx->qro.on;
        ctx->fso.on = ctx->qro.on = false;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
    }
    ~TuneScope()
    {
        ctx->out_tro = out_t;
        ctx->out_qmod = out_q;
        ctx->out_flux = out_f;
        ctx->fso.on = fso_on;
        ctx->qro.on = qro_on;
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
    }
    int copy_states(bool save)
    {
        const size_t M = ctx->M, L = ctx->L;
        if (save) {
            rout = ctx->proc_rout >= 1 && L > 0;
            n_cells_st = M * n_state_planes(ctx->H) * ctx->N;
            n_rt = rout ? 4 * M * L : 0;
            CK(keep.ensure(n_cells_st + n_rt), "autotune state copy");
        }
        double *const rt[4] = {ctx->qtin1.p, ctx->qtr1.p, ctx->qout_last.p, ctx->qmod_last.p};
        CK(cudaMemcpyAsync(save ? keep.p : ctx->states.p, save ? ctx->states.p : keep.p, n_cells_st * sizeof(double),
                           cudaMemcpyDeviceToDevice, ctx->stream),
           "state copy");
        for (int i = 0; rout && i < 4; ++i)
            CK(cudaMemcpyAsync(save ? keep.p + n_cells_st + i * M * L : rt[i],
                               save ? rt[i] : keep.p + n_cells_st + i * M * L, M * L * sizeof(double),
                               cudaMemcpyDeviceToDevice, ctx->stream),
               "state copy");
        return MHM_OK;
    }
    // one trial from the kept states; *ms = its duration
    int trial(int32_t tt0, int32_t n_steps, float *ms)
    {
        if (int rc = copy_states(false)) return rc;
        cudaEventRecord(e0, ctx->stream);
        if (int rc = run_enqueue(ctx, tt0, n_steps, nullptr)) return rc;
        if (int rc = mhm_sync(ctx)) return rc;
        cudaEventRecord(e1, ctx->stream);
        if (cudaEventSynchronize(e1) != cudaSuccess) return fail(ctx, MHM_ERR_CUDA, "autotune timing");
        cudaEventElapsedTime(ms, e0, e1);
        return MHM_OK;
    }
    // the states as they were, once all trials are done
    int finish(int rc)
    {
        if (int r2 = copy_states(false)) rc = rc ? rc : r2;
        if (int r3 = mhm_sync(ctx)) rc = rc ? rc : r3;
        return rc;
    }
};

int mhm_autotune_ex(mhm_ctx *ctx, int32_t tt0, int32_t n_steps, int32_t n_chunk_choices, const int32_t *chunk_choices,
                    mhm_launch_config *best_out, double *ms_out)
{
    NvtxRange nvtx_("mhm: autotune");
    if (!ctx || n_steps < 1 || n_chunk_choices < 0 || n_chunk_choices > 8 ||
        (n_chunk_choices > 0 && !chunk_choices))
        return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc;
    const bool rout = ctx->proc_rout >= 1 && ctx->L > 0;
    const int32_t occ0 = ctx->cell_occ, sub0 = ctx->route_sub, cap0 = ctx->chunk_cap;
    TuneScope ts(ctx);
    int rc = ts.copy_states(true);
    const int occs[3] = {4, 6, 8}, subs[3] = {4, 8, 16};
    std::vector<int32_t> caps = {cap0};
    for (int i = 0; i < n_chunk_choices; ++i) caps.push_back(std::max<int32_t>(0, chunk_choices[i]));
    if (n_chunk_choices > 0) caps.erase(caps.begin());
    const int nc = (int)caps.size(), n_trials = 9 * nc;
    float best = 1e30f;
    int best_occ = occ0, best_sub = sub0, best_cap = cap0;
    // untimed warm-ups first, so that no timed trial pays a first use: module
    // loading of each kernel variant and the capture of each routing graph
    // (every routing sub-chunk with every chunk length)
    std::vector<int> warm;
    for (int c = 0; c < nc; ++c)
        for (int j = 0; j < 3; ++j) warm.push_back(c * 9 + j);     // (4, sub) for each chunk length
    warm.push_back(3);                                            // (6, 4)
    warm.push_back(6);                                            // (8, 4)
    const int nw = (int)warm.size();
    for (int trial = -nw; rc == MHM_OK && trial < n_trials; ++trial) {
        const int ti = trial < 0 ? warm[trial + nw] : trial;
        const int c = ti / 9, v = ti % 9;
        ctx->cell_occ = occs[v / 3];
        ctx->route_sub = rout ? subs[v % 3] : sub0;
        ctx->chunk_cap = caps[c];
        if (!rout && v % 3 != 0) {
            if (trial >= 0 && ms_out) ms_out[trial] = -1.0;
            continue;
        }
        float ms = 0.f;
        if ((rc = ts.trial(tt0, n_steps, &ms))) break;
        if (trial >= 0 && ms_out) ms_out[trial] = ms;
        if (trial >= 0 && ms < best) {
            best = ms;
            best_occ = ctx->cell_occ;
            best_sub = ctx->route_sub;
            best_cap = ctx->chunk_cap;
        }
    }
    ctx->cell_occ = rc == MHM_OK ? best_occ : occ0;
    ctx->route_sub = rc == MHM_OK ? best_sub : sub0;
    ctx->chunk_cap = rc == MHM_OK ? best_cap : cap0;
    rc = ts.finish(rc);
    if (best_out) mhm_get_launch_config(ctx, best_out);
    return rc;
}

int mhm_autotune_route(mhm_ctx *ctx, int32_t tt0, int32_t n_steps, int32_t *cluster_out, double *ms_out)
{
    NvtxRange nvtx_("mhm: autotune routing");
    if (!ctx || n_steps < 1) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc;
    const int32_t modes[4] = {0, 4, 8, 16};
    const int32_t mode0 = ctx->route_cluster;
    int rc = MHM_OK;
    int32_t best_mode = mode0;
    if (ctx->proc_rout >= 1 && ctx->L > 1) {
        TuneScope ts(ctx);
        rc = ts.copy_states(true);
        float best = 1e30f;
        for (int trial = -4; rc == MHM_OK && trial < 4; ++trial) { // one untimed pass over the modes first
            ctx->route_cluster = modes[trial < 0 ? trial + 4 : trial];
            float ms = 0.f;
            if ((rc = ts.trial(tt0, n_steps, &ms))) break;
            if (trial < 0) continue;
            if (ms_out) ms_out[trial] = ms;
            if (ms < best) {
                best = ms;
                best_mode = ctx->route_cluster;
            }
        }
        ctx->route_cluster = rc == MHM_OK ? best_mode : mode0;
        rc = ts.finish(rc);
    } else if (ms_out) {
        for (int i = 0; i < 4; ++i) ms_out[i] = -1.0;
    }
    if (cluster_out) *cluster_out = ctx->route_cluster;
    return rc;
}

int mhm_autotune(mhm_ctx *ctx, int32_t tt0, int32_t n_steps, int32_t *occ_out, int32_t *sub_out, double *ms_out)
{
    if (!ctx) return MHM_ERR_INVALID;
    mhm_launch_config b{};
    const int rc = mhm_autotune_ex(ctx, tt0, n_steps, 0, nullptr, &b, ms_out);
    if (occ_out) *occ_out = b.cell_blocks_per_sm;
    if (sub_out) *sub_out = b.route_sub_steps;
    return rc;
}

int mhm_run(mhm_ctx *ctx, int32_t tt0, int32_t n_steps, double *q_gauge)
{
    if (!ctx) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    int rc = run_enqueue(ctx, tt0, n_steps, q_gauge);
    int rs = mhm_sync(ctx);
    return rc ? rc : rs;
}

int mhm_member_status(mhm_ctx *ctx, int32_t *status)
{
    if (!ctx || !status) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc; // flags of all enqueued steps
    const size_t M = ctx->M;
    std::vector<int32_t> f(M, 0);
    CK(cudaMemcpy(f.data(), ctx->nonfinite.p, M * sizeof(int32_t), cudaMemcpyDeviceToHost), "member flags");
    CK(cudaMemset(ctx->nonfinite.p, 0, M * sizeof(int32_t)), "member flags");
    std::string bad;
    for (size_t m = 0; m < M; ++m) {
        status[m] = f[m] ? MHM_ERR_NAN : MHM_OK;
        if (f[m]) bad += (bad.empty() ? "" : ", ") + std::to_string(m);
    }
    if (!bad.empty()) return fail(ctx, MHM_ERR_NAN, "non-finite state or runoff in member(s) " + bad);
    return MHM_OK;
}

int mhm_enable_fluxes(mhm_ctx *ctx, int32_t on)
{
    if (!ctx) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc;
    ctx->out_flux = on ? 1 : 0;
    if (!on) {
        for (auto &b : ctx->flux_d) b.release();
        ctx->host_aet.clear();
        ctx->host_loss.clear();
    }
    return MHM_OK;
}

int mhm_get_fluxes(mhm_ctx *ctx, double *aet, double *loss)
{
    if (!ctx) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc;
    if (!ctx->out_flux) return fail(ctx, MHM_ERR_INVALID, "flux outputs are not enabled");
    if (aet) std::memcpy(aet, ctx->host_aet.data(), ctx->host_aet.size() * sizeof(double));
    if (loss) std::memcpy(loss, ctx->host_loss.data(), ctx->host_loss.size() * sizeof(double));
    return MHM_OK;
}

int mhm_enable_flux_state_outputs(mhm_ctx *ctx, const mhm_output_config *cfg)
{
    if (!ctx) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc;
    OutSet &o = ctx->fso;
    o.on = false;
    o.acc.release();
    o.out.release();
    o.slots = o.cnt = 0;
    o.slot_tt.clear();
    if (!cfg) return MHM_OK;
    if (cfg->max_slots < 1) return fail(ctx, MHM_ERR_INVALID, "max_slots >= 1 required");
    if (cfg->flags[OF_NEUTRONS - 1])
        return fail(ctx, MHM_ERR_UNSUPPORTED, "neutron output (process 10) is not part of this build");
    // planes in the order of mHM_OutputDataset, src/mHM/mo_write_fluxes_states.f90:82-262
    static const int order[kOutFlags] = {OF_INTERC, OF_SNOW, OF_SWC, OF_SM, OF_SM_ALL, OF_SEAL, OF_UNSAT,
                                         OF_SAT, OF_NEUTRONS, OF_PET, OF_AET, OF_Q, OF_QD, OF_QIF, OF_QIS,
                                         OF_QB, OF_RECHARGE, OF_INFIL, OF_AET_L, OF_PRE_EFFECT, OF_QSM};
    int n = 0;
    uint64_t avg = 0;
    for (int i = 0; i <= kOutFlags; ++i) ctx->fs_plane[i] = -1;
    for (int f : order) {
        if (!cfg->flags[f - 1]) continue;
        const bool per_h = f == OF_SWC || f == OF_SM || f == OF_INFIL || f == OF_AET_L;
        const bool state = f <= OF_SAT; // states are written as interval means (avg = .true.)
        ctx->fs_plane[f] = (int8_t)n;
        for (int j = 0; j < (per_h ? ctx->H : 1); ++j, ++n)
            if (state) avg |= (uint64_t)1 << n;
    }
    if (n == 0) return MHM_OK;
    const size_t MN = (size_t)ctx->M * ctx->N;
    CK(o.acc.ensure((size_t)n * MN), "output sums");
    CK(o.out.ensure((size_t)cfg->max_slots * n * MN), "output intervals");
    CK(cudaMemsetAsync(o.acc.p, 0, (size_t)n * MN * sizeof(double), ctx->stream), "output sums");
    if (!ctx->w_tt.p) {
        std::vector<int64_t> none(ctx->M, -1);
        CK(upload(ctx->w_tt, none.data(), none.size(), ctx->stream), "output weights");
        CK(ctx->w_fs.ensure(MN), "output weights");
        CK(ctx->w_sms.ensure(MN * ctx->H), "output weights");
        CK(cudaStreamSynchronize(ctx->stream), "sync");
    }
    ctx->fs_avg = avg;
    o.n_planes = n;
    o.interval = cfg->timestep_model_outputs;
    o.max_slots = cfg->max_slots;
    o.warm = cfg->warming_steps;
    o.n_tt = cfg->n_time_steps;
    o.on = true;
    return MHM_OK;
}

int mhm_enable_routed_outputs(mhm_ctx *ctx, const mhm_output_config *cfg)
{
    if (!ctx) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc;
    OutSet &o = ctx->qro;
    o.on = false;
    o.acc.release();
    o.out.release();
    o.slots = o.cnt = 0;
    o.slot_tt.clear();
    if (!cfg || !cfg->flags[0]) return MHM_OK;
    if (ctx->proc_rout < 1) return fail(ctx, MHM_ERR_INVALID, "routing is off");
    if (cfg->flags[1]) return fail(ctx, MHM_ERR_UNSUPPORTED, "river temperature (process 11) is not part of this build");
    if (cfg->max_slots < 1) return fail(ctx, MHM_ERR_INVALID, "max_slots >= 1 required");
    const size_t ML = (size_t)ctx->M * ctx->L;
    CK(o.acc.ensure(ML), "Qrouted sums");
    CK(o.out.ensure((size_t)cfg->max_slots * ML), "Qrouted intervals");
    CK(cudaMemsetAsync(o.acc.p, 0, ML * sizeof(double), ctx->stream), "Qrouted sums");
    CK(cudaStreamSynchronize(ctx->stream), "sync");
    o.n_planes = 1;
    o.interval = cfg->timestep_model_outputs;
    o.max_slots = cfg->max_slots;
    o.warm = cfg->warming_steps;
    o.n_tt = cfg->n_time_steps;
    o.on = true;
    return MHM_OK;
}

int mhm_set_output_weights(mhm_ctx *ctx, int32_t m, int64_t tt, const double *fsealed, const double *soil_moist_sat)
{
    if (!ctx) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (m < 0 || m >= ctx->M) return fail(ctx, MHM_ERR_INVALID, "member out of range");
    if (!ctx->fso.on) return fail(ctx, MHM_ERR_INVALID, "flux/state outputs are not enabled");
    if (tt >= 1 && (!fsealed || !soil_moist_sat)) return fail(ctx, MHM_ERR_INVALID, "weights missing");
    if (int rc = mhm_sync(ctx)) return rc;
    const size_t N = ctx->N;
    if (tt >= 1) {
        CK(cudaMemcpy(ctx->w_fs.p + m * N, fsealed, N * sizeof(double), cudaMemcpyHostToDevice), "weights");
        CK(cudaMemcpy(ctx->w_sms.p + (size_t)m * ctx->H * N, soil_moist_sat, (size_t)ctx->H * N * sizeof(double),
                      cudaMemcpyHostToDevice),
           "weights");
    }
    const int64_t v = tt >= 1 ? tt : -1;
    CK(cudaMemcpy(ctx->w_tt.p + m, &v, sizeof(int64_t), cudaMemcpyHostToDevice), "weights");
    return MHM_OK;
}

int mhm_read_flux_state_outputs(mhm_ctx *ctx, double *out, int64_t *slot_tt, int32_t max_slots, int32_t *n_slots,
                                int32_t *n_planes)
{
    if (!ctx) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (n_planes) *n_planes = ctx->fso.on ? ctx->fso.n_planes : 0;
    return read_outset(ctx, ctx->fso, out, slot_tt, max_slots, n_slots, false);
}

int mhm_read_routed_outputs(mhm_ctx *ctx, double *out, int64_t *slot_tt, int32_t max_slots, int32_t *n_slots)
{
    if (!ctx) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    return read_outset(ctx, ctx->qro, out, slot_tt, max_slots, n_slots, true);
}

int mhm_get_state(mhm_ctx *ctx, int32_t m, const mhm_restart *st)
{
    if (!ctx || !st) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (m < 0 || m >= ctx->M) return fail(ctx, MHM_ERR_INVALID, "member out of range");
    if (int rc = mhm_sync(ctx)) return rc; // states of all enqueued steps
    const size_t N = ctx->N, L = ctx->L;
    const int H = ctx->H, ns = n_state_planes(H);
    const double *S = ctx->states.p + (size_t)m * ns * N;
    double *dst[5] = {st->interc, st->snowpack, st->sealSTW, st->unsatSTW, st->satSTW};
    const int pl[5] = {S_INTERC, S_SNOW, S_SEAL, S_UNSAT, S_SAT};
    for (int i = 0; i < 5; ++i)
        if (dst[i]) CK(cudaMemcpy(dst[i], S + (size_t)pl[i] * N, N * sizeof(double), cudaMemcpyDeviceToHost), "state");
    if (st->soilMoist)
        CK(cudaMemcpy(st->soilMoist, S + (size_t)S_SM * N, (size_t)H * N * sizeof(double), cudaMemcpyDeviceToHost),
           "SM");
    if (ctx->proc_rout >= 1) {
        std::vector<double> buf(L);
        auto by_node = [&](const double *dev, double *out, size_t off) -> int {
            CK(cudaMemcpy(buf.data(), dev + m * L, L * sizeof(double), cudaMemcpyDeviceToHost), "routing state");
            for (size_t v = 0; v < L; ++v) out[off + v] = buf[ctx->net.pos_of_node[v]];
            return MHM_OK;
        };
        int rc;
        if (st->qOUT && (rc = by_node(ctx->qout_last.p, st->qOUT, 0))) return rc;
        if (st->Qmod && (rc = by_node(ctx->qmod_last.p, st->Qmod, 0))) return rc;
        if (st->qTIN) {
            if ((rc = by_node(ctx->qtin1.p, st->qTIN, 0))) return rc;
            std::memcpy(st->qTIN + L, st->qTIN, L * sizeof(double));
        }
        if (st->qTR) {
            if ((rc = by_node(ctx->qtr1.p, st->qTR, 0))) return rc;
            std::memcpy(st->qTR + L, st->qTR, L * sizeof(double));
        }
        // L11_C1 / L11_C2 are per link (1..nLinks), the tail stays at its initial 0
        auto by_link = [&](const double *dev, double *out) -> int {
            CK(cudaMemcpy(buf.data(), dev + m * L, L * sizeof(double), cudaMemcpyDeviceToHost), "routing coeffs");
            for (size_t i = 0; i < L; ++i) out[i] = 0.0;
            for (int i = 0; i < ctx->n_links; ++i) out[i] = buf[ctx->net.link_pos[i]];
            return MHM_OK;
        };
        if (st->C1 && (rc = by_link(ctx->C1.p, st->C1))) return rc;
        if (st->C2 && (rc = by_link(ctx->C2.p, st->C2))) return rc;
    }
    return MHM_OK;
}

int mhm_set_state(mhm_ctx *ctx, int32_t m, const mhm_restart *st)
{
    if (!ctx || !st) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (m < 0 || m >= ctx->M) return fail(ctx, MHM_ERR_INVALID, "member out of range");
    if (int rc = mhm_sync(ctx)) return rc;
    const size_t N = ctx->N, L = ctx->L;
    const int H = ctx->H, ns = n_state_planes(H);
    double *S = ctx->states.p + (size_t)m * ns * N;
    const double *src[5] = {st->interc, st->snowpack, st->sealSTW, st->unsatSTW, st->satSTW};
    const int pl[5] = {S_INTERC, S_SNOW, S_SEAL, S_UNSAT, S_SAT};
    for (int i = 0; i < 5; ++i)
        if (src[i]) CK(cudaMemcpy(S + (size_t)pl[i] * N, src[i], N * sizeof(double), cudaMemcpyHostToDevice), "state");
    if (st->soilMoist)
        CK(cudaMemcpy(S + (size_t)S_SM * N, st->soilMoist, (size_t)H * N * sizeof(double), cudaMemcpyHostToDevice),
           "SM");
    if (ctx->proc_rout >= 1) {
        std::vector<double> buf(L);
        auto to_pos = [&](const double *in, double *dev) -> int {
            for (size_t v = 0; v < L; ++v) buf[ctx->net.pos_of_node[v]] = in[v];
            CK(cudaMemcpy(dev + m * L, buf.data(), L * sizeof(double), cudaMemcpyHostToDevice), "routing state");
            return MHM_OK;
        };
        int rc;
        if (st->qOUT && (rc = to_pos(st->qOUT, ctx->qout_last.p))) return rc;
        if (st->Qmod && (rc = to_pos(st->Qmod, ctx->qmod_last.p))) return rc;
        if (st->qTIN && (rc = to_pos(st->qTIN, ctx->qtin1.p))) return rc;
        if (st->qTR && (rc = to_pos(st->qTR, ctx->qtr1.p))) return rc;
        auto link_to_pos = [&](const double *in, double *dev) -> int {
            std::fill(buf.begin(), buf.end(), 0.0);
            for (int i = 0; i < ctx->n_links; ++i) buf[ctx->net.link_pos[i]] = in[i];
            CK(cudaMemcpy(dev + m * L, buf.data(), L * sizeof(double), cudaMemcpyHostToDevice), "routing coeffs");
            return MHM_OK;
        };
        if (st->C1 && (rc = link_to_pos(st->C1, ctx->C1.p))) return rc;
        if (st->C2 && (rc = link_to_pos(st->C2, ctx->C2.p))) return rc;
    }
    return MHM_OK;
}

int mhm_get_var(mhm_ctx *ctx, int32_t m, const char *name, double *out)
{
    if (!ctx || !name || !out) return MHM_ERR_INVALID;
    mhm_restart st{};
    const std::string n(name);
    if (n == "L1_INTER") st.interc = out;
    else if (n == "L1_SNOWPACK") st.snowpack = out;
    else if (n == "L1_SEALSTW") st.sealSTW = out;
    else if (n == "L1_SOILMOIST") st.soilMoist = out;
    else if (n == "L1_UNSATSTW") st.unsatSTW = out;
    else if (n == "L1_SATSTW") st.satSTW = out;
    else if (n == "L11_QMOD") st.Qmod = out;
    else if (n == "L11_QOUT") st.qOUT = out;
    else return fail(ctx, MHM_ERR_INVALID, "unknown variable " + n);
    if ((st.Qmod || st.qOUT) && ctx->proc_rout < 1) return fail(ctx, MHM_ERR_INVALID, "routing is off");
    return mhm_get_state(ctx, m, &st);
}

int mhm_set_timing(mhm_ctx *ctx, int32_t on)
{
    if (!ctx) return MHM_ERR_INVALID;
    ctx->timing = on != 0;
    for (int i = 0; i < 4; ++i) {
        ctx->t_launches[i] = 0;
        ctx->t_ms[i] = 0.0;
    }
    return MHM_OK;
}

int mhm_get_timing(mhm_ctx *ctx, int32_t kind, int64_t *launches, double *total_ms)
{
    if (!ctx || kind < 0 || kind > 3) return MHM_ERR_INVALID;
    if (launches) *launches = ctx->t_launches[kind];
    if (total_ms) *total_ms = ctx->t_ms[kind];
    return MHM_OK;
}

int mhm_routing_order(int32_t n_nodes, int32_t n_outlets, const int32_t *from_n, const int32_t *to_n,
                      int32_t *net_perm, int32_t *r_order)
{
    if (n_nodes < 1 || n_outlets < 0 || n_outlets > n_nodes || !from_n || !to_n || !net_perm || !r_order)
        return MHM_ERR_INVALID;
    std::string err;
    if (!routing_order(n_nodes, n_outlets, from_n, to_n, net_perm, r_order, err)) {
        std::fprintf(stderr, "mhm_routing_order: %s\n", err.c_str());
        return MHM_ERR_INVALID;
    }
    return MHM_OK;
}

int mhm_l11_network_size(int32_t nrows0, int32_t ncols0, const uint8_t *mask0, int32_t factor, int32_t *n_nodes)
{
    if (nrows0 < 1 || ncols0 < 1 || factor < 1 || !mask0 || !n_nodes) return MHM_ERR_INVALID;
    const int32_t nr11 = (nrows0 + factor - 1) / factor, nc11 = (ncols0 + factor - 1) / factor;
    std::vector<char> m((size_t)nr11 * nc11, 0);
    for (int32_t j = 0; j < ncols0; ++j)
        for (int32_t i = 0; i < nrows0; ++i)
            if (mask0[(size_t)j * nrows0 + i]) m[(size_t)(j / factor) * nr11 + i / factor] = 1;
    int32_t n = 0;
    for (char c : m) n += c ? 1 : 0;
    *n_nodes = n;
    return MHM_OK;
}

int mhm_l11_network(const mhm_l0_flow *in, mhm_l11_network_out *out)
{
    NvtxRange nvtx_("mhm: network start-up");
    if (!in || !out || !in->mask0 || !in->fdir0 || !in->facc0 || !in->elev0 || in->n_cells0 < 1 ||
        !(in->cellsize0 > 0.0) || in->n_lc_scenes < 0 || (in->n_lc_scenes > 0 && !in->lcover0))
        return MHM_ERR_INVALID;
    L0FlowInput li;
    li.nrows0 = in->nrows0;
    li.ncols0 = in->ncols0;
    li.factor = in->factor;
    li.n_cells0 = in->n_cells0;
    li.mask0 = in->mask0;
    li.fdir0 = in->fdir0;
    li.facc0 = in->facc0;
    li.elev0 = in->elev0;
    li.cellsize0 = in->cellsize0;
    li.n_lc_scenes = in->n_lc_scenes;
    li.lc_class_imp = in->lc_class_imp;
    li.lcover0 = in->lcover0;
    L11NetworkOut o;
    std::string err;
    if (!build_l11_network(li, o, err)) {
        std::fprintf(stderr, "mhm_l11_network: %s\n", err.c_str());
        return MHM_ERR_INVALID;
    }
    out->n_nodes = o.n_nodes;
    out->n_outlets = o.n_outlets;
    out->n_links = o.n_links;
    out->nrows11 = o.nrows11;
    out->ncols11 = o.ncols11;
    out->n_l0_outlets = o.n_l0_outlets;
    auto put_i = [](int32_t *dst, const std::vector<int32_t> &v) {
        if (dst) std::memcpy(dst, v.data(), v.size() * sizeof(int32_t));
    };
    auto put_d = [](double *dst, const std::vector<double> &v) {
        if (dst) std::memcpy(dst, v.data(), v.size() * sizeof(double));
    };
    put_i(out->fdir11, o.fdir11);
    put_i(out->cell_row11, o.cell_row11);
    put_i(out->cell_col11, o.cell_col11);
    put_i(out->from_n, o.from_n);
    put_i(out->to_n, o.to_n);
    put_i(out->net_perm, o.net_perm);
    put_i(out->r_order, o.r_order);
    put_i(out->row_out, o.row_out);
    put_i(out->col_out, o.col_out);
    put_d(out->length, o.length);
    put_d(out->slope, o.slope);
    put_d(out->a_floodplain, o.a_floodplain);
    put_d(out->frac_fp_imp, o.frac_fp_imp);
    return MHM_OK;
}

int mhm_l1_l11_mapping(int32_t nrows0, int32_t ncols0, const uint8_t *mask0, int32_t factor1, int32_t factor11,
                       int32_t *l1_l11_id, int32_t *l11_l1_id)
{
    if (!mask0) return MHM_ERR_INVALID;
    std::vector<int32_t> a, b;
    std::string err;
    if (!l1_l11_mapping(nrows0, ncols0, mask0, factor1, factor11, a, b, err)) {
        std::fprintf(stderr, "mhm_l1_l11_mapping: %s\n", err.c_str());
        return MHM_ERR_INVALID;
    }
    if (l1_l11_id) std::memcpy(l1_l11_id, a.data(), a.size() * sizeof(int32_t));
    if (l11_l1_id) std::memcpy(l11_l1_id, b.data(), b.size() * sizeof(int32_t));
    return MHM_OK;
}

int mhm_network_topology(int32_t nrows, int32_t ncols, const int32_t *id2d, int32_t n_cells, const int32_t *cell_row,
                         const int32_t *cell_col, const int32_t *fdir, int32_t *from_n, int32_t *to_n,
                         int32_t *n_links)
{
    if (nrows < 1 || ncols < 1 || n_cells < 1 || !id2d || !cell_row || !cell_col || !fdir || !from_n || !to_n ||
        !n_links)
        return MHM_ERR_INVALID;
    std::string err;
    if (!network_topology(nrows, ncols, id2d, n_cells, cell_row, cell_col, fdir, from_n, to_n, n_links, err)) {
        std::fprintf(stderr, "mhm_network_topology: %s\n", err.c_str());
        return MHM_ERR_INVALID;
    }
    return MHM_OK;
}

int mhm_step_calendar(int32_t jul_start, int32_t timestep, int32_t tt0, int32_t n, int32_t *month,
                      int32_t *hour, int32_t *doy)
{
    if (jul_start < 2299161 || timestep < 1 || 24 % timestep != 0 || tt0 < 1 || n < 0) return MHM_ERR_INVALID;
    for (int32_t i = 0; i < n; ++i) {
        StepDate sd = step_date(jul_start, timestep, (int64_t)tt0 + i);
        if (month) month[i] = sd.month;
        if (hour) hour[i] = sd.hour;
        if (doy) doy[i] = sd.doy;
    }
    return MHM_OK;
}

int mhm_step_lai(int32_t jul_start, int32_t timestep, int32_t lai_mode, int32_t tt0, int32_t n, int32_t *lai)
{
    if (jul_start < 2299161 || timestep < 1 || 24 % timestep != 0 || tt0 < 1 || n < 0 || lai_mode < -3 ||
        lai_mode > 1 || (n > 0 && !lai))
        return MHM_ERR_INVALID;
    for (int32_t i = 0; i < n; ++i) lai[i] = step_lai(jul_start, timestep, (int64_t)tt0 + i, lai_mode);
    return MHM_OK;
}

int mhm_gamma_layout(int32_t proc_soilmoist, int32_t proc_pet, int32_t proc_routing, int32_t n_geo_units,
                     int32_t *offsets)
{
    GammaOffsets o{};
    if (!offsets || !gamma_layout(proc_soilmoist, proc_pet, proc_routing, n_geo_units, o)) return MHM_ERR_INVALID;
    const int32_t v[11] = {o.interc, o.snow, o.soil, o.runoff, o.pet, o.interflow, o.perc, o.routing, o.geo,
                           o.total, o.total};
    std::memcpy(offsets, v, sizeof(v));
    return MHM_OK;
}

int mhm_mpr_setup(mhm_ctx *ctx, const mhm_l0_desc *l0)
{
    NvtxRange nvtx_("mhm: MPR set-up");
    if (!ctx || !l0) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc;
    ctx->mpr_ready = false;
    if (ctx->proc_pet < -1 || ctx->proc_pet > 3)
        return fail(ctx, MHM_ERR_UNSUPPORTED, "MPR supports PET cases -1 to 3");
    if (l0->max_soil_hor > kMprMaxSoilHor)
        return fail(ctx, MHM_ERR_UNSUPPORTED, "more than 16 soil layers per soil type");
    MprSetup &m = ctx->mpr;
    m = MprSetup{};
    std::string err;
    if (!mpr_prepare(*l0, ctx->N, ctx->H, m, err)) return fail(ctx, MHM_ERR_INVALID, err);
    const size_t slots = (size_t)m.max_sub * m.n1, nsh = (size_t)m.n_soil * m.max_hor;
    std::vector<double> soil;
    soil.reserve(3 * nsh + m.n_soil + m.Wd.size() + m.H);
    soil.insert(soil.end(), m.sand.begin(), m.sand.end());
    soil.insert(soil.end(), m.clay.begin(), m.clay.end());
    soil.insert(soil.end(), m.dbm.begin(), m.dbm.end());
    soil.insert(soil.end(), m.rz.begin(), m.rz.end());
    soil.insert(soil.end(), m.Wd.begin(), m.Wd.end());
    soil.insert(soil.end(), m.horizon_depth.begin(), m.horizon_depth.end());
    std::vector<double> frac;
    frac.reserve(4 * (size_t)m.n1);
    for (const auto *v : {&m.f_forest, &m.f_sealed, &m.f_perm, &m.f_kar}) frac.insert(frac.end(), v->begin(), v->end());
    cudaStream_t s = ctx->stream;
    CK(upload(ctx->mpr_nhor, m.n_hor.data(), m.n_hor.size(), s), "mpr soil");
    CK(upload(ctx->mpr_ntill, m.n_till.data(), m.n_till.size(), s), "mpr soil");
    CK(upload(ctx->mpr_nsub, m.nsub.data(), m.nsub.size(), s), "mpr nsub");
    CK(upload(ctx->mpr_code, m.sub_code.data(), slots, s), "mpr codes");
    CK(upload(ctx->mpr_soil, soil.data(), soil.size(), s), "mpr soil");
    CK(upload(ctx->mpr_se, m.sub_se.data(), slots, s), "mpr slope");
    CK(upload(ctx->mpr_asp, m.sub_asp.data(), slots, s), "mpr aspect");
    CK(upload(ctx->mpr_frac, frac.data(), frac.size(), s), "mpr fractions");
    if (m.n_lai_classes > 0) {
        CK(upload(ctx->mpr_lut, m.lai_lut.data(), m.lai_lut.size(), s), "mpr LAI");
        ctx->mpr_lai.release();
    } else {
        CK(upload(ctx->mpr_lai, m.sub_lai.data(), m.sub_lai.size(), s), "mpr LAI");
        CK(ctx->mpr_lut.ensure(1), "mpr LAI");
    }
    CK(cudaStreamSynchronize(s), "mpr setup");
    ctx->mpr_ready = true;
    return MHM_OK;
}

int mhm_mpr(mhm_ctx *ctx, int32_t member0, int32_t n, const double *gammas, int32_t n_gamma)
{
    NvtxRange nvtx_("mhm: MPR");
    if (!ctx || !gammas) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (int rc = mhm_sync(ctx)) return rc; // no enqueued step may still read the parameters
    if (!ctx->mpr_ready) return fail(ctx, MHM_ERR_INVALID, "mhm_mpr_setup has not been called");
    if (n < 1 || member0 < 0 || member0 + n > ctx->M) return fail(ctx, MHM_ERR_INVALID, "members out of range");
    const MprSetup &m = ctx->mpr;
    GammaOffsets off{};
    if (!gamma_layout(ctx->proc_sm, ctx->proc_pet, ctx->proc_rout, m.n_geo, off))
        return fail(ctx, MHM_ERR_INVALID, "no parameter layout for these processes");
    if (n_gamma != off.total)
        return fail(ctx, MHM_ERR_INVALID,
                    "parameter vector has " + std::to_string(n_gamma) + " entries, expected " + std::to_string(off.total));
    cudaStream_t s = ctx->stream;
    const int ts = mpr_table_stride(ctx->H);
    const size_t slots = (size_t)m.max_sub * m.n1, nsh = (size_t)m.n_soil * m.max_hor;
    CK(upload(ctx->mpr_gamma, gammas, (size_t)n * n_gamma, s), "parameters");
    CK(ctx->mpr_table.ensure((size_t)n * m.n_keys * ts), "mpr table");
    CK(ctx->mpr_petlai.ensure(std::max<size_t>(1, (size_t)n * 3 * m.n_lai_classes * 12)), "mpr table");
    MprArgs a{};
    a.n1 = m.n1;
    a.max_sub = m.max_sub;
    a.H = ctx->H;
    a.proc_sm = ctx->proc_sm;
    a.proc_pet = ctx->proc_pet;
    a.n_soil = m.n_soil;
    a.max_hor = m.max_hor;
    a.n_keys = m.n_keys;
    a.n_lai_classes = m.n_lai_classes;
    a.n_gamma = n_gamma;
    a.n_members = n;
    a.off = off;
    a.dpth_t_last = m.dpth_t_last;
    a.n_hor = ctx->mpr_nhor.p;
    a.n_till = ctx->mpr_ntill.p;
    const double *sp = ctx->mpr_soil.p;
    a.sand = sp;
    a.clay = sp + nsh;
    a.dbm = sp + 2 * nsh;
    a.rz = sp + 3 * nsh;
    a.Wd = a.rz + m.n_soil;
    a.hd = a.Wd + m.Wd.size();
    a.lai_lut = ctx->mpr_lut.p;
    a.nsub = ctx->mpr_nsub.p;
    a.code = ctx->mpr_code.p;
    a.se = ctx->mpr_se.p;
    a.asp = ctx->mpr_asp.p;
    a.lai = (m.n_lai_classes > 0) ? nullptr : ctx->mpr_lai.p;
    a.f_forest = ctx->mpr_frac.p;
    a.f_sealed = a.f_forest + m.n1;
    a.f_perm = a.f_sealed + m.n1;
    a.f_kar = a.f_perm + m.n1;
    a.gamma = ctx->mpr_gamma.p;
    a.table = ctx->mpr_table.p;
    a.petlai = ctx->mpr_petlai.p;
    const int64_t np = n_param_planes(ctx->H);
    a.member_stride = np * ctx->N;
    a.params = ctx->params.p + (size_t)member0 * a.member_stride;
    (void)slots;
    if (int rc = mpr_lai_target(ctx, m, member0, a)) return rc;
    CK(launch_mpr(a, s), "mpr");
    g_launches += 2;
    if (ctx->proc_rout == 1 && ctx->n_links > 0) {
        const size_t L = ctx->L;
        for (int32_t i = 0; i < n; ++i) {
            const int32_t mm = member0 + i;
            const double *p5 = ctx->mpr_gamma.p + (size_t)i * n_gamma + off.routing;
            CK(cudaMemcpyAsync(ctx->rout_p5.p + 5 * mm, p5, 5 * sizeof(double), cudaMemcpyDeviceToDevice, s), "p5");
            CK(launch_reg_rout(ctx->n_links, ctx->rout_p5.p + 5 * mm, ctx->ss_max, (double)ctx->timestep,
                               ctx->length.p, ctx->slope.p, ctx->ffp.p, ctx->link_pos.p, ctx->C1.p + mm * L,
                               ctx->C2.p + mm * L, s),
               "reg_rout");
            g_launches++;
        }
    }
    if (ctx->proc_rout == 2)
        for (int32_t i = 0; i < n; ++i)
            if (int rc = set_adaptive_member(ctx, member0 + i, gammas[(size_t)i * n_gamma + off.routing], nullptr))
                return rc;
    CK(cudaStreamSynchronize(s), "mpr sync");
    return MHM_OK;
}

// mhm_mpr for one member without any device allocation.  mhm_mpr keeps its
// parameter vectors and soil tables in context buffers that grow with the
// number of members per call, i.e. it may cudaMalloc/cudaFree.  Callers that
// must not do that use this variant: a serving loop or calibration driver
// that sized its device memory once up front and runs several contexts side
// by side -- cudaMalloc can fail once that budget is taken, and cudaFree may
// synchronise the whole device, stalling the other contexts' streams.  Here
// the per-call data live in g_mpr_scratch, whose address is looked up once
// per device (cudaGetSymbolAddress, with the device current); all other
// buffers were allocated by mhm_ctx_create and mhm_mpr_setup.
//
// Nothing in the scratch has to start at zero: the parameter vector is
// copied in first, and every table entry the upscaling reads is written by
// the table kernel earlier on the same stream.  The scratch is shared by all
// contexts on a device, so two calls whose work overlaps (from two host
// threads, or on different contexts' streams) race on it; the call
// synchronises its stream before returning, so consecutive calls from one
// thread are safe.  The first call on a device performs the address lookup,
// which may load the module: make that first call before any stream capture
// begins on the device.
int mhm_mpr_noalloc(mhm_ctx *ctx, int32_t member, const double *gamma, int32_t n_gamma)
{
    NvtxRange nvtx_("mhm: MPR (static scratch)");
    if (!ctx || !gamma) return MHM_ERR_INVALID;
    ON_CTX_DEVICE(ctx);
    if (!ctx->mpr_ready) return fail(ctx, MHM_ERR_INVALID, "mhm_mpr_setup has not been called");
    if (member < 0 || member >= ctx->M) return fail(ctx, MHM_ERR_INVALID, "member out of range");
    if (ctx->proc_rout >= 2) return fail(ctx, MHM_ERR_UNSUPPORTED, "adaptive routing: use mhm_mpr");
    const MprSetup &m = ctx->mpr;
    GammaOffsets off{};
    if (!gamma_layout(ctx->proc_sm, ctx->proc_pet, ctx->proc_rout, m.n_geo, off))
        return fail(ctx, MHM_ERR_INVALID, "no parameter layout for these processes");
    if (n_gamma != off.total) return fail(ctx, MHM_ERR_INVALID, "parameter vector length does not match the layout");
    const int ts = mpr_table_stride(ctx->H);
    // the LAI-correction table is used only by PET case -1 with class LAI
    const size_t n_table = (size_t)m.n_keys * ts;
    const size_t n_petlai = (ctx->proc_pet == -1 && m.n_lai_classes > 0) ? (size_t)3 * m.n_lai_classes * 12 : 0;
    const size_t need = align32((size_t)n_gamma) + align32(n_table) + n_petlai;
    if (need > kMprScratchDoubles)
        return fail(ctx, MHM_ERR_INVALID,
                    "mhm_mpr_noalloc needs " + std::to_string(need) + " doubles of scratch; the static scratch holds " +
                        std::to_string(kMprScratchDoubles) + " (512 KiB): use mhm_mpr");
    if (ctx->device < 0 || ctx->device >= kMaxScratchDevices)
        return fail(ctx, MHM_ERR_UNSUPPORTED, "device ordinal beyond the scratch address table");
    double *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mu);
        if (!g_scratch_addr[ctx->device]) {
            void *p = nullptr;
            CK(cudaGetSymbolAddress(&p, g_mpr_scratch), "scratch address");
            g_scratch_addr[ctx->device] = static_cast<double *>(p);
        }
        scratch = g_scratch_addr[ctx->device];
    }
    cudaStream_t s = ctx->stream;
    // after every step already enqueued on this context (cell chain on
    // `stream`, routing on `route_stream`) has read the old parameters
    CK(cudaEventRecord(ctx->ev_route_end, ctx->route_stream), "record route end");
    CK(cudaStreamWaitEvent(s, ctx->ev_route_end, 0), "join");
    double *d_gamma = scratch;
    double *d_table = scratch + align32((size_t)n_gamma);
    double *d_petlai = d_table + align32(n_table);
    CK(cudaMemcpyAsync(d_gamma, gamma, (size_t)n_gamma * sizeof(double), cudaMemcpyHostToDevice, s), "parameters");
    const size_t nsh = (size_t)m.n_soil * m.max_hor;
    MprArgs a{};
    a.n1 = m.n1;
    a.max_sub = m.max_sub;
    a.H = ctx->H;
    a.proc_sm = ctx->proc_sm;
    a.proc_pet = ctx->proc_pet;
    a.n_soil = m.n_soil;
    a.max_hor = m.max_hor;
    a.n_keys = m.n_keys;
    a.n_lai_classes = m.n_lai_classes;
    a.n_gamma = n_gamma;
    a.n_members = 1;
    a.off = off;
    a.dpth_t_last = m.dpth_t_last;
    a.n_hor = ctx->mpr_nhor.p;
    a.n_till = ctx->mpr_ntill.p;
    a.sand = ctx->mpr_soil.p;
    a.clay = a.sand + nsh;
    a.dbm = a.sand + 2 * nsh;
    a.rz = a.sand + 3 * nsh;
    a.Wd = a.rz + m.n_soil;
    a.hd = a.Wd + m.Wd.size();
    a.lai_lut = ctx->mpr_lut.p;
    a.nsub = ctx->mpr_nsub.p;
    a.code = ctx->mpr_code.p;
    a.se = ctx->mpr_se.p;
    a.asp = ctx->mpr_asp.p;
    a.lai = (m.n_lai_classes > 0) ? nullptr : ctx->mpr_lai.p;
    a.f_forest = ctx->mpr_frac.p;
    a.f_sealed = a.f_forest + m.n1;
    a.f_perm = a.f_sealed + m.n1;
    a.f_kar = a.f_perm + m.n1;
    a.gamma = d_gamma;
    a.table = d_table;
    a.petlai = d_petlai;
    a.member_stride = (int64_t)n_param_planes(ctx->H) * ctx->N;
    a.params = ctx->params.p + (size_t)member * a.member_stride;
    if (int rc = mpr_lai_target(ctx, m, member, a)) return rc;
    CK(launch_mpr(a, s), "mpr");
    g_launches += 2;
    if (ctx->proc_rout == 1 && ctx->n_links > 0) {
        const size_t L = ctx->L;
        CK(cudaMemcpyAsync(ctx->rout_p5.p + 5 * member, d_gamma + off.routing, 5 * sizeof(double),
                           cudaMemcpyDeviceToDevice, s),
           "p5");
        CK(launch_reg_rout(ctx->n_links, ctx->rout_p5.p + 5 * member, ctx->ss_max, (double)ctx->timestep,
                           ctx->length.p, ctx->slope.p, ctx->ffp.p, ctx->link_pos.p, ctx->C1.p + member * L,
                           ctx->C2.p + member * L, s),
           "reg_rout");
        g_launches++;
    }
    CK(cudaStreamSynchronize(s), "mpr sync");
    return MHM_OK;
}

int mhm_soil_weights(int32_t n_soil, int32_t max_hor, const int32_t *n_hor, const double *ud, const double *ld,
                     const double *rz_depth, int32_t n_h, double *horizon_depth, double *wd)
{
    if (n_soil < 1 || max_hor < 1 || n_h < 1 || !n_hor || !ud || !ld || !rz_depth || !horizon_depth || !wd)
        return MHM_ERR_INVALID;
    std::string err;
    return soil_weights(n_soil, max_hor, n_hor, ud, ld, rz_depth, n_h, horizon_depth, wd, err) ? MHM_OK
                                                                                              : MHM_ERR_INVALID;
}

int mhm_slope_emp(int32_t n, const double *slope, double *slope_emp)
{
    if (n < 0 || (n > 0 && (!slope || !slope_emp))) return MHM_ERR_INVALID;
    slope_empirical(n, slope, slope_emp);
    return MHM_OK;
}

int mhm_mpr_get_aux(mhm_ctx *ctx, const char *name, double *out)
{
    if (!ctx || !name || !out) return MHM_ERR_INVALID;
    if (!ctx->mpr_ready) return fail(ctx, MHM_ERR_INVALID, "mhm_mpr_setup has not been called");
    const std::vector<double> *v = nullptr;
    if (!std::strcmp(name, "Wd")) v = &ctx->mpr.Wd;
    else if (!std::strcmp(name, "slope_emp")) v = &ctx->mpr.slope_emp;
    else if (!std::strcmp(name, "horizon_depth")) v = &ctx->mpr.horizon_depth;
    if (!v) return fail(ctx, MHM_ERR_INVALID, std::string("unknown MPR start-up product ") + name);
    std::memcpy(out, v->data(), v->size() * sizeof(double));
    return MHM_OK;
}

int mhm_host_alloc(size_t bytes, void **ptr)
{
    if (!ptr) return MHM_ERR_INVALID;
    cudaError_t e = cudaHostAlloc(ptr, bytes, cudaHostAllocPortable);
    return e == cudaSuccess ? MHM_OK : (e == cudaErrorMemoryAllocation ? MHM_ERR_OOM : MHM_ERR_CUDA);
}

int mhm_host_free(void *ptr)
{
    return cudaFreeHost(ptr) == cudaSuccess ? MHM_OK : MHM_ERR_CUDA;
}

int mhm_hmath_eval(int32_t op, int32_t where, int64_t n, const double *x, const double *y, double *out)
{
    if (op < 0 || op > 3 || n < 0 || !x || !out || (op >= 2 && !y)) return MHM_ERR_INVALID;
    if (where == 0) {
        for (int64_t i = 0; i < n; ++i)
            out[i] = op == 0 ? hm_log(x[i]) : op == 1 ? hm_exp(x[i]) : op == 2 ? hm_pow(x[i], y[i]) : hm_div(x[i], y[i]);
        return MHM_OK;
    }
    double *dx = nullptr, *dy = nullptr, *dout = nullptr;
    auto cleanup = [&]() {
        cudaFree(dx);
        cudaFree(dy);
        cudaFree(dout);
    };
    size_t bytes = (size_t)n * sizeof(double);
    if (cudaMalloc(&dx, bytes) != cudaSuccess || cudaMalloc(&dout, bytes) != cudaSuccess ||
        (op >= 2 && cudaMalloc(&dy, bytes) != cudaSuccess)) {
        cleanup();
        return MHM_ERR_OOM;
    }
    cudaMemcpy(dx, x, bytes, cudaMemcpyHostToDevice);
    if (op >= 2) cudaMemcpy(dy, y, bytes, cudaMemcpyHostToDevice);
    cudaError_t e = launch_hmath_eval(op, n, dx, dy, dout, 0);
    g_launches++;
    if (e == cudaSuccess) e = cudaMemcpy(out, dout, bytes, cudaMemcpyDeviceToHost);
    cleanup();
    return e == cudaSuccess ? MHM_OK : MHM_ERR_CUDA;
}

int mhm_batch_create(int32_t device, mhm_batch **out)
{
    if (!out) return MHM_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return MHM_ERR_CUDA;
    int cur = 0;
    if (device < 0 && cudaGetDevice(&cur) != cudaSuccess) cur = 0;
    if (device >= ndev) return MHM_ERR_INVALID;
    mhm_batch *b = new mhm_batch();
    b->device = device >= 0 ? device : cur;
    if (const char *s = std::getenv("MHM_FUSED_OCC")) b->occ = std::atoi(s) >= 8 ? 8 : 4;
    DeviceGuard dg(b->device);
    if (dg.err != cudaSuccess || cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_done, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&b->ev_staged, cudaEventDisableTiming) != cudaSuccess ||
        b->queue.ensure(1) != cudaSuccess) {
        mhm_batch_destroy(b);
        return MHM_ERR_CUDA;
    }
    *out = b;
    return MHM_OK;
}

int mhm_batch_destroy(mhm_batch *b)
{
    if (!b) return MHM_OK;
    DeviceGuard dg(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    for (cudaEvent_t e : b->ev_pre)
        if (e) cudaEventDestroy(e);
    if (b->ev_done) cudaEventDestroy(b->ev_done);
    if (b->ev_staged) cudaEventDestroy(b->ev_staged);
    if (b->h_args) cudaFreeHost(b->h_args);
    if (b->h_tile_ctx) cudaFreeHost(b->h_tile_ctx);
    if (b->h_item0) cudaFreeHost(b->h_item0);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return MHM_OK;
}

const char *mhm_batch_last_error(const mhm_batch *b) { return b ? b->err.c_str() : "null batch"; }

int mhm_batch_run_members(mhm_batch *b, int32_t n, mhm_ctx *const *ctxs, const int32_t *const *member_tt0,
                          int32_t n_steps, double *const *q_gauge)
{
    NvtxRange nvtx_("mhm: fused batch round");
    if (!b || n < 1 || !ctxs || !member_tt0 || n_steps < 1) return MHM_ERR_INVALID;
    auto bfail = [&](int code, const std::string &m) {
        b->err = m;
        return code;
    };
    DeviceGuard dg(b->device);
    if (dg.err != cudaSuccess) return bfail(MHM_ERR_CUDA, "set device");
    bool lean = false;
    int hmax = 1;
    for (int32_t i = 0; i < n; ++i) {
        mhm_ctx *c = ctxs[i];
        if (!c || !member_tt0[i]) return bfail(MHM_ERR_INVALID, "context or member steps missing");
        for (int32_t j = 0; j < i; ++j)
            if (ctxs[j] == c) return bfail(MHM_ERR_INVALID, "a context appears twice");
        if (c->device != b->device) return bfail(MHM_ERR_INVALID, "context on another device than the batch");
        if (c->out_tro || c->out_qmod || c->out_flux || c->fso.on || c->qro.on)
            return bfail(MHM_ERR_UNSUPPORTED, "per-step or aggregated outputs in a fused launch");
        const bool l = (c->proc_pet == 0 || c->proc_pet == -1) && (c->proc_sm == 1 || c->proc_sm == 4);
        if (i > 0 && l != lean) return bfail(MHM_ERR_UNSUPPORTED, "contexts with different process code paths");
        lean = l;
        hmax = std::max(hmax, c->H);
    }
    const int hl = hmax <= 6 ? 6 : 8;
    if ((int)b->ev_pre.size() < n) {
        const size_t old = b->ev_pre.size();
        b->ev_pre.resize(n, nullptr);
        for (size_t i = old; i < (size_t)n; ++i)
            if (cudaEventCreateWithFlags(&b->ev_pre[i], cudaEventDisableTiming) != cudaSuccess)
                return bfail(MHM_ERR_CUDA, "event");
    }
    // phase 1: every context enqueues its call up to the cell chain
    std::vector<FusedStage> fs(n);
    for (int32_t i = 0; i < n; ++i) {
        mhm_ctx *c = ctxs[i];
        fs[i].phase = 1;
        if (int rc = run_enqueue(c, 1, n_steps, q_gauge ? q_gauge[i] : nullptr, member_tt0[i], &fs[i]))
            return bfail(rc, "context " + std::to_string(i) + ": " + c->err);
        if (cudaEventRecord(b->ev_pre[i], c->stream) != cudaSuccess ||
            cudaStreamWaitEvent(b->stream, b->ev_pre[i], 0) != cudaSuccess)
            return bfail(MHM_ERR_CUDA, "event");
    }
    // the work queue: tiles of 128 items, contexts with more horizons first
    std::vector<int32_t> order(n);
    for (int32_t i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) {
        return ctxs[x]->H > ctxs[y]->H ||
               (ctxs[x]->H == ctxs[y]->H && (int64_t)ctxs[x]->N * ctxs[x]->M > (int64_t)ctxs[y]->N * ctxs[y]->M);
    });
    size_t n_tiles = 0;
    for (int32_t i = 0; i < n; ++i) n_tiles += ((size_t)ctxs[i]->N * ctxs[i]->M + 127) / 128;
    if (n_tiles > (size_t)INT32_MAX) return bfail(MHM_ERR_UNSUPPORTED, "too many tiles");
    if (b->staged && cudaEventSynchronize(b->ev_staged) != cudaSuccess) return bfail(MHM_ERR_CUDA, "staging");
    if (b->cap_ctx < (size_t)n) {
        if (b->h_args) cudaFreeHost(b->h_args);
        b->h_args = nullptr;
        b->cap_ctx = 0;
        if (cudaMallocHost((void **)&b->h_args, (size_t)n * sizeof(CellArgs)) != cudaSuccess)
            return bfail(MHM_ERR_OOM, "staging");
        b->cap_ctx = n;
    }
    if (b->cap_tiles < n_tiles) {
        if (b->h_tile_ctx) cudaFreeHost(b->h_tile_ctx);
        if (b->h_item0) cudaFreeHost(b->h_item0);
        b->h_tile_ctx = nullptr;
        b->h_item0 = nullptr;
        b->cap_tiles = 0;
        if (cudaMallocHost((void **)&b->h_tile_ctx, n_tiles * sizeof(int32_t)) != cudaSuccess ||
            cudaMallocHost((void **)&b->h_item0, n_tiles * sizeof(int64_t)) != cudaSuccess)
            return bfail(MHM_ERR_OOM, "staging");
        b->cap_tiles = n_tiles;
    }
    size_t t = 0;
    for (int32_t oi = 0; oi < n; ++oi) {
        const int32_t i = order[oi];
        b->h_args[i] = fs[i].args;
        const int64_t items = (int64_t)ctxs[i]->N * ctxs[i]->M;
        for (int64_t it = 0; it < items; it += 128, ++t) {
            b->h_tile_ctx[t] = i;
            b->h_item0[t] = it;
        }
    }
    if (b->args.ensure(n) != cudaSuccess || b->tile_ctx.ensure(n_tiles) != cudaSuccess ||
        b->tile_item0.ensure(n_tiles) != cudaSuccess)
        return bfail(MHM_ERR_OOM, "batch tables");
    if (cudaMemcpyAsync(b->args.p, b->h_args, (size_t)n * sizeof(CellArgs), cudaMemcpyHostToDevice, b->stream) ||
        cudaMemcpyAsync(b->tile_ctx.p, b->h_tile_ctx, n_tiles * sizeof(int32_t), cudaMemcpyHostToDevice, b->stream) ||
        cudaMemcpyAsync(b->tile_item0.p, b->h_item0, n_tiles * sizeof(int64_t), cudaMemcpyHostToDevice, b->stream) ||
        cudaMemsetAsync(b->queue.p, 0, sizeof(int32_t), b->stream) || cudaEventRecord(b->ev_staged, b->stream))
        return bfail(MHM_ERR_CUDA, "batch tables upload");
    b->staged = true;
    FusedCellArgs f{};
    f.args = b->args.p;
    f.tile_ctx = b->tile_ctx.p;
    f.tile_item0 = b->tile_item0.p;
    f.n_tiles = (int32_t)n_tiles;
    f.queue = b->queue.p;
    if (cudaError_t e = launch_cell_chain_fused(f, hl, lean, b->occ, b->stream))
        return bfail(MHM_ERR_CUDA, std::string("fused cell chain: ") + cudaGetErrorString(e));
    g_launches++;
    if (cudaEventRecord(b->ev_done, b->stream) != cudaSuccess) return bfail(MHM_ERR_CUDA, "event");
    b->rounds += 1;
    b->tiles_total += (int64_t)n_tiles;
    // phase 2: the rest of every context's call, after the fused cell chain
    for (int32_t i = 0; i < n; ++i) {
        fs[i].phase = 2;
        fs[i].ev_fused = b->ev_done;
        if (int rc = run_enqueue(ctxs[i], 1, n_steps, q_gauge ? q_gauge[i] : nullptr, member_tt0[i], &fs[i]))
            return bfail(rc, "context " + std::to_string(i) + ": " + ctxs[i]->err);
    }
    return MHM_OK;
}

int mhm_probe_fp64(int64_t iters, double *flops)
{
    if (iters < 1 || !flops) return MHM_ERR_INVALID;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return MHM_ERR_CUDA;
    const int threads = 256, blocks = sms * 8;
    double *sink = nullptr;
    if (cudaMalloc(&sink, (size_t)blocks * threads * sizeof(double)) != cudaSuccess) return MHM_ERR_OOM;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    launch_fp64_probe(iters / 10 + 1, blocks, threads, sink, 0); // warm-up
    cudaEventRecord(a, 0);
    cudaError_t e = launch_fp64_probe(iters, blocks, threads, sink, 0);
    cudaEventRecord(b, 0);
    g_launches += 2;
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    cudaFree(sink);
    if (e != cudaSuccess || ms <= 0.f) return MHM_ERR_CUDA;
    // 8 independent chains per thread, 1 DFMA (2 FLOP) each per iteration
    *flops = 2.0 * 8.0 * (double)iters * blocks * threads / (ms * 1e-3);
    return MHM_OK;
}

} // extern "C"
