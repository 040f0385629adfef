// batch_fast.cu - the batched sweep kernels under the fast math
// policy (batch_kernel.cuh).
#include "batch_kernel.cuh"

namespace mhd {

cudaError_t launch_batch_sweep_fast(const SweepWork &w, bool rows, int grid, int threads, size_t smem,
                                        cudaStream_t s)
{
    return rows ? launch_batch_sweep_inst<Fast, true>(w, grid, threads, smem, s)
                : launch_batch_sweep_inst<Fast, false>(w, grid, threads, smem, s);
}

int batch_sweep_occupancy_fast(bool rows, int threads, size_t smem)
{
    return rows ? batch_sweep_occupancy_inst<Fast, true>(threads, smem)
                : batch_sweep_occupancy_inst<Fast, false>(threads, smem);
}

}  // namespace mhd
