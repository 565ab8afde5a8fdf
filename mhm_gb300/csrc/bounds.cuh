// bounds.cuh -- index checks of the bounds-checked build (-DMHM_BOUNDS_CHECK).
//
// Every index a kernel takes from data rather than from its thread index --
// forcing rows of the calendar, the member step table, network tables, L1
// <-> L11 mappings, gauge and inflow positions, inflow days, entries of a
// gridded LAI series, soil keys, LAI classes and geology units of the L0
// codes -- is tested before the access.
// A failed test records (site, index) in the translation unit's device status
// word (the first failure wins, atomicCAS) and the access is skipped; nothing
// traps, so the context stays usable and the host reports the failure
// (mhm_device_status, mhm_sync).  Other builds compile the tests away.
#pragma once
#include <cstdint>

#include <cuda_runtime.h>

namespace mhm {

enum BoundsSite : int {
    BC_FORCING_ROW = 1,  // cell chain: forcing row of the step in the forcing window
    BC_STEP_ROW = 2,     // cell chain (member mode): row of the member step table
    BC_ACC_CELL = 3,     // runoff accumulation: L1 cell of a node
    BC_ACC_L1 = 4,       // runoff accumulation: the L1 cell of an L11 cell (L11 finer than L1)
    BC_ROUTE_UP = 5,     // routing: upstream position
    BC_ROUTE_QOUT = 6,   // routing: qOUT row of a routing step
    BC_GAUGE_POS = 7,    // gauge gather: gauge position
    BC_INFLOW_POS = 8,   // add_inflow: inflow gauge position
    BC_INFLOW_DAY = 9,   // add_inflow: day of the inflow discharge series
    BC_MPR_KEY = 10,     // MPR: soil key of an L0 cell
    BC_MPR_LAI = 11,     // MPR: LAI class of an L0 cell
    BC_MPR_GEO = 12,     // MPR: geology unit of an L0 cell
    BC_LAI_STEP = 13,    // cell chain: entry of a gridded LAI series
    BC_SELFTEST = 99,    // mhm_bounds_selftest
};

// (site << 48) | (index & 0xffffffffffff) of the first failed test, 0 = none;
// one word per translation unit (and per device)
static __device__ unsigned long long g_bc_status;

#if defined(MHM_BOUNDS_CHECK)
constexpr bool kBoundsChecked = true;
__device__ __forceinline__ bool bc_ok(int site, long long i, long long n)
{
    if (i >= 0 && i < n) return true;
    const unsigned long long v =
        ((unsigned long long)(site & 0xffff) << 48) | ((unsigned long long)i & 0xffffffffffffULL);
    atomicCAS(&g_bc_status, 0ull, v);
    return false;
}
#else
constexpr bool kBoundsChecked = false;
__device__ __forceinline__ bool bc_ok(int, long long, long long) { return true; }
#endif

// host: read and clear this translation unit's status word on the current device
static inline cudaError_t bc_take_word(unsigned long long *out)
{
    cudaError_t e = cudaMemcpyFromSymbol(out, g_bc_status, sizeof(unsigned long long));
    if (e != cudaSuccess || *out == 0) return e;
    const unsigned long long zero = 0;
    return cudaMemcpyToSymbol(g_bc_status, &zero, sizeof(zero));
}

} // namespace mhm

// one exported reader per translation unit that launches checked kernels
#define MHM_BC_ACCESSOR(name)                                                                                \
    namespace mhm {                                                                                           \
    cudaError_t name(unsigned long long *out) { return bc_take_word(out); }                                   \
    }
