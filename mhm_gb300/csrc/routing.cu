// routing.cu -- mRM L1->L11 runoff accumulation and Muskingum link routing,
// time-chunked and level-synchronous.
//
// The reference advances every link one step at a time in netPerm order
// (L11_routing, src/mRM/mo_mrm_routing.f90:380-481).  The per-link recurrence
// only reads the link's own previous step and the same-step outflow of its
// upstream links, so a whole chunk of steps of one link can run as soon as the
// chunk of every upstream link is done: links are grouped into topological
// levels and each level advances its links through the full chunk.  Inflow
// sums at confluences keep the reference's order (upstream links in netPerm
// rank order, then the node's own qOUT), so results are bit-identical.
#include <atomic>
#include <cstdint>

#include "bounds.cuh"
#include "calendar.h"
#include "mhm_kernels.cuh"

namespace mhm {

// L11_runoff_acc, src/mRM/mo_mrm_pre_routing.f90:77-143: per (step, member,
// node) the area-weighted sum of its L1 cells in ascending cell order, then
// *1000/TST.  Output indexed by routing-level position.
__global__ void __launch_bounds__(256) runoff_acc_kernel(const AccArgs a)
{
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t L = a.n_nodes;
    const int64_t total = (int64_t)a.n_steps * a.n_members * L;
    if (gid >= total) return;
    const int pos = (int)(gid % L);
    const int64_t tm = gid / L; // t * M + m
    const int m = (int)(tm % a.n_members);
    const int t = (int)(tm / a.n_members);
    if (a.member_step0 && a.member_step0[m] < 0) return; // idle member
    // runoff of cell k for routing step t: the model step's value, or with a
    // routing step of `win` model steps their sum from 0 in step order
    // (RunToRout, src/mHM/mo_mhm_interface_run.f90:489-490)
    const size_t row_stride = (size_t)a.n_members * a.n_cells;
    const double *row = a.tro + ((size_t)t * a.win * a.n_members + m) * a.n_cells;
    auto run = [&](int k) -> double {
        if (a.win == 1) return __ldg(row + k);
        double r = 0.0;
        for (int j = 0; j < a.win; ++j) r = r + __ldg(row + j * row_stride + k);
        return r;
    };
    double q;
    if (a.map_flag) {
        double acc = 0.0;
        const int b = __ldg(a.node_cell_ptr + pos), e = __ldg(a.node_cell_ptr + pos + 1);
        for (int j = b; j < e; ++j) {
            const int k = __ldg(a.node_cells + j);
            if (!bc_ok(BC_ACC_CELL, k, a.n_cells)) continue;
            acc = acc + run(k) * __ldg(a.l1_area + k);
        }
        q = acc * 1000.0 / a.TST;
    } else {
        const int k = __ldg(a.pos_l11_l1 + pos);
        q = bc_ok(BC_ACC_L1, k, a.n_cells) ? run(k) * __ldg(a.pos_area + pos) * 1000.0 / a.TST : 0.0;
    }
    a.qout[((size_t)m * a.n_steps + t) * L + pos] = q;
}

// One (member, node) of a wavefront tick: the node advances its sub-chunk
// (tick - level) of `sub` <= SUB steps.  L11_routing body,
// src/mRM/mo_mrm_routing.f90:435-478.  Inflow sums keep the reference order:
// per step, ((0 + qTR(up_1)) + qTR(up_2) + ...) + qOUT, upstream links in
// netPerm rank order; the upstream series of the whole sub-chunk are loaded
// first (independent loads), then the Muskingum recurrence runs.  Everything
// another thread wrote in an earlier tick (routed outflow, node states) is
// read through L2 (ld.global.cg), so the function is also correct where
// consecutive ticks run in one launch on different SMs.
template <int SUB>
__device__ __forceinline__ void route_item(const RouteArgs &a, const int m, const int pos, const int tick)
{
    // the item's own words first, all in flight together (every index is in
    // range for any member and position; only the upstream reads depend on them)
    const int64_t L = a.n_nodes;
    const size_t ms = (size_t)m * L;
    const int level = __ldg(a.pos_level + pos);
    const int ub = __ldg(a.up_ptr + pos), ue = __ldg(a.up_ptr + pos + 1);
    const int flags = __ldg(a.pos_flags + pos);
    double qtin1 = __ldcg(a.qtin1 + ms + pos);
    double qtr1 = __ldcg(a.qtr1 + ms + pos);
    const double c1 = __ldg(a.C1 + ms + pos);
    const double c2 = __ldg(a.C2 + ms + pos);
    if (a.member_step0 && a.member_step0[m] < 0) return; // idle member: routing states untouched
    const int s = tick - level;
    const int t0 = s * a.sub;
    if (s < 0 || t0 >= a.n_steps) return;
    const int nt = min(a.sub, a.n_steps - t0);
    const size_t base = ((size_t)m * a.n_steps + t0) * L; // row t0 of member m
    const bool is_link = flags & 1;
    const bool add_qout = flags & 2;
    const bool cut = flags & 4; // mo_mrm_routing.f90:447-452
    double qtin[SUB];
#pragma unroll
    for (int t = 0; t < SUB; ++t) qtin[t] = 0.0; // netNode_qTIN(:, IT) = 0
    for (int j = ub; j < ue; ++j) {
        const int up_pos = __ldg(a.up_pos + j);
        if (!bc_ok(BC_ROUTE_UP, up_pos, L)) continue;
        const double *up = a.qtr + base + up_pos;
#pragma unroll
        for (int t = 0; t < SUB; ++t)
            if (t < nt) qtin[t] = qtin[t] + __ldcg(up + (size_t)t * L);
    }
    if (add_qout && bc_ok(BC_ROUTE_QOUT, (t0 + nt - 1) / a.rdiv, a.n_qsteps)) {
        const double *qo = a.qout + (size_t)m * a.n_qsteps * L + pos;
#pragma unroll
        for (int t = 0; t < SUB; ++t)
            if (t < nt) qtin[t] = qtin[t] + __ldcg(qo + (size_t)((t0 + t) / a.rdiv) * L);
    }
#pragma unroll
    for (int t = 0; t < SUB; ++t) {
        if (t < nt) {
            const size_t row = base + (size_t)t * L;
            if (is_link) {
                double qtr = qtr1 + c1 * (qtin1 - qtr1) + c2 * (qtin[t] - qtin1);
                if (cut) qtr = 0.0;
                a.qtr[row + pos] = qtr;
                qtr1 = qtr;
            }
            qtin1 = qtin[t];
            a.qmod[row + pos] = 0.0 + qtin[t]; // L11_qMod = (0 + Qmod) / real(rout_loop = 1)
        }
    }
    a.qtin1[ms + pos] = qtin1;
    a.qtr1[ms + pos] = qtr1;
}

// One wavefront tick per launch: threads over (member, position) of the
// levels the tick spans.
template <int SUB>
__global__ void __launch_bounds__(128) route_tick_kernel(const RouteArgs a)
{
    const int width = a.pos_end - a.pos_begin;
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (int64_t)width * a.n_members) return;
    const int m = (int)(gid / width);
    route_item<SUB>(a, m, a.pos_begin + (int)(gid - (int64_t)m * width), a.tick);
}

// All ticks of a chunk in one launch: each thread-block cluster walks the
// wavefront of its members (m = cluster, cluster + clusters, ...), its CTAs
// sharing the (member, position) items of a tick, with a hardware cluster
// barrier between ticks.  The CTAs of a cluster are co-scheduled by the
// hardware and every thread reaches every barrier (no thread leaves the tick
// loop early), so no wait depends on work outside the cluster; clusters never
// wait on one another.  The barrier's release/acquire orders a tick's stores
// before the next tick's L2 reads.
__device__ __forceinline__ unsigned cluster_sreg_rank()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cluster_sreg_size()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cluster_sreg_id()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%clusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cluster_sreg_count()
{
    unsigned r;
    asm volatile("mov.u32 %0, %%nclusterid.x;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_barrier()
{
    asm volatile("barrier.cluster.arrive.release;\n\tbarrier.cluster.wait.acquire;" ::: "memory");
}

// 512 threads per CTA: one item per thread in the ticks of a 62,500-node
// network on a 16-CTA cluster (measured: 128 / 256 / 512 threads took 21.7 /
// 17.6 / 16.2 ms for its 240-step chunk)
constexpr int kWalkThreads = 512;

template <int SUB>
__global__ void __launch_bounds__(kWalkThreads) route_walk_kernel(const RouteArgs a, const RouteWalk w)
{
    const int cs = (int)cluster_sreg_size(), rank = (int)cluster_sreg_rank();
    const int cid = (int)cluster_sreg_id(), ncl = (int)cluster_sreg_count();
    // items interleaved over the CTAs (item i on CTA i % cs): a tick's work
    // spreads over every SM of the cluster, whose FP64 pipes bound it
    const int nthr = cs * (int)blockDim.x;
    const int tid = (int)threadIdx.x * cs + rank;
    const int mc = cid < a.n_members ? (a.n_members - cid + ncl - 1) / ncl : 0; // this cluster's members
    for (int k = 0; k < w.n_ticks; ++k) {
        const int lo = max(0, k - w.n_sub + 1), hi = min(k, w.n_levels - 1);
        const int pb = __ldg(w.level_ptr + lo), pe = __ldg(w.level_ptr + hi + 1);
        const int width = pe - pb;
        const int items = width * mc; // < 2^31: positions x members of one context
        for (int i = tid; i < items; i += nthr) {
            const int mi = i / width;
            route_item<SUB>(a, cid + mi * ncl, pb + (i - mi * width), k);
        }
        cluster_barrier();
    }
}

__global__ void inflow_kernel(const InflowArgs a)
{
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (gid >= (int64_t)a.n_members * a.n_qsteps) return;
    const int m = (int)(gid / a.n_qsteps), s = (int)(gid - (int64_t)m * a.n_qsteps);
    int64_t tt0 = a.tt_base;
    if (a.member_step0) {
        const int32_t b = a.member_step0[m];
        if (b < 0) return; // idle member
        tt0 = (int64_t)b + a.step_shift + 1;
    }
    tt0 += (int64_t)s * a.win; // first model step of routing step s
    double *row = a.qout + ((size_t)m * a.n_qsteps + s) * a.n_nodes;
    // the days of this routing step (the host checks that the series covers the run)
    const int64_t d_first = (tt0 + a.steps_day - 1) / a.steps_day - a.day0;
    const int64_t d_last = (tt0 + (a.mean ? a.win - 1 : 0) + a.steps_day - 1) / a.steps_day - a.day0;
    if (!bc_ok(BC_INFLOW_DAY, d_first, a.n_days) || !bc_ok(BC_INFLOW_DAY, d_last, a.n_days)) return;
    for (int g = 0; g < a.n_inflow; ++g) {
        double Q;
        if (a.mean) {
            double acc = 0.0;
            for (int j = 0; j < a.win; ++j) {
                const int64_t day = (tt0 + j + a.steps_day - 1) / a.steps_day;
                acc = acc + __ldg(a.q + (size_t)(day - a.day0) * a.n_inflow + g);
            }
            Q = acc / a.tsf;
        } else {
            const int64_t day = (tt0 + a.steps_day - 1) / a.steps_day;
            Q = __ldg(a.q + (size_t)(day - a.day0) * a.n_inflow + g);
        }
        const int p = __ldg(a.pos + g);
        if (!bc_ok(BC_INFLOW_POS, p, a.n_nodes)) continue;
        double *v = row + p;
        *v = a.headwater[g] ? *v + Q : Q;
    }
}

// mhm_bounds_selftest: one failing test (index == extent) with no access
// behind it, so that the status path can be checked without any bad access
__global__ void bc_selftest_kernel(int n) { bc_ok(BC_SELFTEST, n, n); }

cudaError_t launch_bc_selftest(cudaStream_t s)
{
    bc_selftest_kernel<<<1, 1, 0, s>>>(7);
    return cudaGetLastError();
}

cudaError_t launch_inflow(const InflowArgs &a, cudaStream_t s)
{
    const int64_t n = (int64_t)a.n_members * a.n_qsteps;
    if (n == 0 || a.n_inflow == 0) return cudaSuccess;
    inflow_kernel<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(a);
    return cudaGetLastError();
}

__global__ void qmod_step_kernel(const QmodStepArgs a)
{
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t L = a.n_nodes;
    if (gid >= (int64_t)a.n_members * a.n_steps * L) return;
    const int pos = (int)(gid % L);
    const int64_t mt = gid / L;
    const int t = (int)(mt % a.n_steps), m = (int)(mt / a.n_steps);
    if (a.member_step0 && a.member_step0[m] < 0) return;
    const int64_t n_sub = (int64_t)a.n_steps * a.rdiv / a.win;
    const double *q = a.qmod_sub + (size_t)m * n_sub * L + pos;
    double v;
    if (a.rdiv > 1) {
        double acc = 0.0;
        for (int r = 0; r < a.rdiv; ++r) acc = acc + q[(size_t)(t * a.rdiv + r) * L];
        v = acc / (double)a.rdiv;
    } else {
        v = q[(size_t)(t / a.win) * L];
    }
    a.qmod[((size_t)m * a.n_steps + t) * L + pos] = v;
}

// mRM's Qrouted output (mRM_updateDataset / writeTimestep, called every model
// step after the warm-up: src/mHM/mo_mhm_interface_run.f90:651-668).  One
// thread per (member, node) walks the chunk's steps; with a routing step of
// `win` model steps the discharge state changes only at a window's last step.
__global__ void qrouted_kernel(const QroutArgs a)
{
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t L = a.n_nodes;
    if (gid >= (int64_t)a.n_members * L) return;
    const int pos = (int)(gid % L);
    const int m = (int)(gid / L);
    const size_t ML = (size_t)a.n_members * L;
    const double *q = a.qmod + (size_t)m * a.n_steps * L + pos;
    double acc = a.acc[(size_t)m * L + pos];
    int cnt = a.cnt0, slot = a.slot0;
    for (int t = 0; t < a.n_steps; ++t) {
        const int64_t tt = a.tt_base + t;
        if (tt <= a.warm_steps) continue;
        double v;
        if (a.win == 1 || (t + 1) % a.win == 0) v = q[(size_t)t * L];
        else if (t >= a.win) v = q[(size_t)((t / a.win) * a.win - 1) * L];
        else v = a.qmod_prev[(size_t)m * L + pos];
        acc = acc + v;
        ++cnt;
        if (out_writeout(a.interval, tt - a.warm_steps, tt, a.n_tt, step_dflags(a.jul_start, a.timestep, tt))) {
            if (slot < a.max_slots) a.out[(size_t)slot * ML + (size_t)m * L + pos] = acc / (double)cnt; // a mean
            acc = 0.0;
            cnt = 0;
            ++slot;
        }
    }
    a.acc[(size_t)m * L + pos] = acc;
}

// GaugeDischarge(gaugeIndexList) = L11_Qmod(gaugeNodeList), mo_mrm_routing.f90:299-301
__global__ void gauge_gather_kernel(const GaugeArgs a)
{
    const int64_t gid = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = (int64_t)a.n_members * a.n_gauges * a.n_steps;
    if (gid >= total) return;
    const int t = (int)(gid % a.n_steps);
    const int64_t mg = gid / a.n_steps;
    const int g = (int)(mg % a.n_gauges);
    const int m = (int)(mg / a.n_gauges);
    const int gp = __ldg(a.gauge_pos + g);
    const double v = (a.member_step0 && a.member_step0[m] < 0) || !bc_ok(BC_GAUGE_POS, gp, a.n_nodes)
                         ? 0.0
                         : a.qmod[((size_t)m * a.n_steps + t) * a.n_nodes + gp];
    a.q_gauge[((size_t)m * a.n_gauges + g) * a.total_steps + a.step_offset + t] = v;
}

// reg_rout, src/mRM/mo_mrm_mpr.f90:61-119, one thread per link; ss_max is the
// basin's max slope (parameter independent, computed on the host once).
__global__ void reg_rout_kernel(int n_links, const double *p5, double ss_max, double TS,
                                const double *length, const double *slope, const double *ffp,
                                const int32_t *link_pos, double *C1, double *C2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_links) return;
    const double p0 = p5[0], p1 = p5[1], p2 = p5[2], p3 = p5[3], p4 = p5[4];
    double K = p0 + p1 * (length[i] * 0.001) + p2 * slope[i] + p3 * ffp[i];
    double xi = p4 * (1.0 + slope[i] / ss_max);
    if (xi > 0.5) xi = 0.5;
    if (xi < 0.005) xi = 0.005;
    if (K > 0.5 * TS / xi) K = 0.5 * TS / xi;
    if (K < 0.5 * TS / (1.0 - xi)) K = 0.5 * TS / (1.0 - xi);
    const double c1 = TS / (K * (1.0 - xi) + 0.5 * TS);
    const int pos = link_pos[i];
    C1[pos] = c1;
    C2[pos] = 1.0 - c1 * K / TS;
}

cudaError_t launch_runoff_acc(const AccArgs &a, cudaStream_t s)
{
    const int64_t n = (int64_t)a.n_steps * a.n_members * a.n_nodes;
    if (n == 0) return cudaSuccess;
    runoff_acc_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_route_tick(const RouteArgs &a, cudaStream_t s)
{
    const int64_t n = (int64_t)(a.pos_end - a.pos_begin) * a.n_members;
    if (n == 0) return cudaSuccess;
    const unsigned grid = (unsigned)((n + 127) / 128);
    if (a.sub <= 4) route_tick_kernel<4><<<grid, 128, 0, s>>>(a);
    else if (a.sub <= 8) route_tick_kernel<8><<<grid, 128, 0, s>>>(a);
    else if (a.sub <= 16) route_tick_kernel<16><<<grid, 128, 0, s>>>(a);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

// Clusters of `cs` CTAs (4, 8 or 16; 16 is a non-portable size, and a size
// no SM group of the device can hold falls back to the next smaller one), at
// most one per member and no more than can be resident at once.  The
// occupancy answer is kept per (device, SUB, cluster size).
template <int SUB>
static cudaError_t launch_route_walk_t(const RouteArgs &a, const RouteWalk &w, int cs, cudaStream_t s)
{
    constexpr int kDevs = 16;
    static std::atomic<int> max_active[kDevs][3] = {}; // 0: not queried yet; -1: does not fit
    auto kern = route_walk_kernel<SUB>;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.blockDim = dim3(kWalkThreads, 1, 1);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    for (; cs >= 4; cs /= 2) {
        const int ci = cs == 4 ? 0 : cs == 8 ? 1 : 2;
        at[0].val.clusterDim.x = (unsigned)cs;
        int mc = dev < kDevs ? max_active[dev][ci].load() : 0;
        if (mc == 0) {
            if (cs > 8) {
                e = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
                if (e != cudaSuccess) return e;
            }
            cfg.gridDim = dim3((unsigned)cs, 1, 1);
            e = cudaOccupancyMaxActiveClusters(&mc, kern, &cfg);
            if (e != cudaSuccess) return e;
            if (mc < 1) mc = -1;
            if (dev < kDevs) max_active[dev][ci].store(mc);
        }
        if (mc < 1) continue;
        const int ncl = a.n_members < mc ? a.n_members : mc;
        cfg.gridDim = dim3((unsigned)(ncl * cs), 1, 1);
        return cudaLaunchKernelEx(&cfg, kern, a, w);
    }
    return cudaErrorInvalidConfiguration;
}

cudaError_t launch_route_walk(const RouteArgs &a, const RouteWalk &w, int cs, cudaStream_t s)
{
    if (a.n_members < 1 || w.n_ticks < 1) return cudaSuccess;
    if (cs != 4 && cs != 8 && cs != 16) return cudaErrorInvalidValue;
    if (a.sub <= 4) return launch_route_walk_t<4>(a, w, cs, s);
    if (a.sub <= 8) return launch_route_walk_t<8>(a, w, cs, s);
    if (a.sub <= 16) return launch_route_walk_t<16>(a, w, cs, s);
    return cudaErrorInvalidValue;
}

cudaError_t launch_qmod_step(const QmodStepArgs &a, cudaStream_t s)
{
    const int64_t n = (int64_t)a.n_members * a.n_steps * a.n_nodes;
    if (n == 0) return cudaSuccess;
    qmod_step_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_qrouted(const QroutArgs &a, cudaStream_t s)
{
    const int64_t n = (int64_t)a.n_members * a.n_nodes;
    if (n == 0 || a.n_steps == 0) return cudaSuccess;
    qrouted_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_gauge_gather(const GaugeArgs &a, cudaStream_t s)
{
    const int64_t n = (int64_t)a.n_members * a.n_gauges * a.n_steps;
    if (n == 0) return cudaSuccess;
    gauge_gather_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_reg_rout(int n_links, const double *p5, double ss_max, double TS, const double *length,
                            const double *slope, const double *ffp, const int32_t *link_pos, double *C1,
                            double *C2, cudaStream_t s)
{
    if (n_links <= 0) return cudaSuccess;
    reg_rout_kernel<<<(n_links + 127) / 128, 128, 0, s>>>(n_links, p5, ss_max, TS, length, slope, ffp, link_pos,
                                                          C1, C2);
    return cudaGetLastError();
}

} // namespace mhm

MHM_BC_ACCESSOR(bc_take_routing)
