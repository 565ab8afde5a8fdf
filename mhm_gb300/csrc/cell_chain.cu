// cell_chain.cu -- launchers of the cell-chain kernel (register variant for
// 4 resident blocks per SM) and of the step-calendar kernel.  Variants sized
// for 6 and 8 resident blocks per SM live in cell_chain_o6.cu / _o8.cu.
#include "cell_chain_impl.cuh"

namespace mhm {

cudaError_t launch_cell_chain_o6(const CellArgs &a, int H, cudaStream_t s);
cudaError_t launch_cell_chain_o8(const CellArgs &a, int H, cudaStream_t s);

// Calendar of steps tt0 .. tt0+n-1: forcing row, month, day flags, day of year.
__global__ void steps_fill_kernel(StepInfo *steps, int64_t tt0, int32_t n, int32_t jul_start, int32_t timestep,
                                  int32_t stride, int32_t lai_mode)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int64_t tt = tt0 + i;
    const StepDate sd = step_date(jul_start, timestep, tt);
    StepInfo si;
    si.row = (int32_t)((tt + stride - 1) / stride); // iMeteoTS, mo_meteo_handler.f90:575-620
    si.month = (int8_t)sd.month;
    si.dflags = (int8_t)step_dflags(jul_start, timestep, tt);
    si.doy = (int16_t)sd.doy;
    si.hour = (int8_t)sd.hour;
    si.lai = (int16_t)step_lai(jul_start, timestep, tt, lai_mode);
    steps[i] = si;
}

cudaError_t launch_steps_fill(StepInfo *steps, int64_t tt0, int32_t n, int32_t jul_start, int32_t timestep,
                              int32_t stride, int32_t lai_mode, cudaStream_t s)
{
    if (n <= 0) return cudaSuccess;
    steps_fill_kernel<<<(n + 255) / 256, 256, 0, s>>>(steps, tt0, n, jul_start, timestep, stride, lai_mode);
    return cudaGetLastError();
}

// The persistent multi-context launch: hl = horizon planes of the shared
// layout (6 or 8, at least every context's horizon count), `lean` as the
// contexts' common code path, occ = resident blocks per SM the registers are
// sized for (4 or 8).  One resident wave of blocks takes the tiles.
cudaError_t launch_cell_chain_fused(const FusedCellArgs &f, int hl, bool lean, int occ, cudaStream_t s)
{
    if (f.n_tiles <= 0) return cudaSuccess;
    const int block = 128;
    const size_t smem = hs_bytes(hl, block);
    void (*k)(const FusedCellArgs) = nullptr;
    const bool o8 = occ >= 8;
    if (hl == 6)
        k = lean ? (o8 ? cell_chain_fused_kernel<6, true, 8> : cell_chain_fused_kernel<6, true, 4>)
                 : (o8 ? cell_chain_fused_kernel<6, false, 8> : cell_chain_fused_kernel<6, false, 4>);
    else if (hl == 8)
        k = lean ? (o8 ? cell_chain_fused_kernel<8, true, 8> : cell_chain_fused_kernel<8, true, 4>)
                 : (o8 ? cell_chain_fused_kernel<8, false, 8> : cell_chain_fused_kernel<8, false, 4>);
    else
        return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, nb = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, block, smem)) != cudaSuccess) return e;
    const int64_t wave = (int64_t)(nb < 1 ? 1 : nb) * sms;
    const unsigned grid = (unsigned)(f.n_tiles < wave ? f.n_tiles : wave);
    k<<<grid, block, smem, s>>>(f);
    return cudaGetLastError();
}

// occ = resident blocks per SM the kernel's registers are sized for (4, 6, 8)
cudaError_t launch_cell_chain(const CellArgs &a, int H, int occ, cudaStream_t s)
{
    if (H < 1 || H > kMaxHorizons) return cudaErrorInvalidValue;
    // per-step fluxes or aggregated outputs: one variant
    if (a.flux_aet || a.out.n_planes > 0) return launch_cell_chain_variant<4, true>(a, H, s);
    switch (occ) {
    case 6: return launch_cell_chain_o6(a, H, s);
    case 8: return launch_cell_chain_o8(a, H, s);
    default: return launch_cell_chain_variant<4>(a, H, s);
    }
}

} // namespace mhm

MHM_BC_ACCESSOR(bc_take_cell_chain)
