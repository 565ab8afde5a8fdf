// cell_chain_o6.cu -- the cell-chain kernel with registers sized for 6
// resident blocks per SM (more warps to hide latency, some values spilled).
#include "cell_chain_impl.cuh"

namespace mhm {

cudaError_t launch_cell_chain_o6(const CellArgs &a, int H, cudaStream_t s)
{
    if (H < 1 || H > kMaxHorizons) return cudaErrorInvalidValue;
    return launch_cell_chain_variant<6>(a, H, s);
}

} // namespace mhm

MHM_BC_ACCESSOR(bc_take_cell_chain_o6)
