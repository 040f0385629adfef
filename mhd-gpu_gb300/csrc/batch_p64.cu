// batch_p64.cu - the batched sweep kernels under the faithful policy
// with FP64 pressure recovery in low-beta cells (batch_kernel.cuh).
#include "batch_kernel.cuh"

namespace mhd {

cudaError_t launch_batch_sweep_p64(const SweepWork &w, bool rows, int grid, int threads, size_t smem,
                                        cudaStream_t s)
{
    return rows ? launch_batch_sweep_inst<Recover64, true>(w, grid, threads, smem, s)
                : launch_batch_sweep_inst<Recover64, false>(w, grid, threads, smem, s);
}

int batch_sweep_occupancy_p64(bool rows, int threads, size_t smem)
{
    return rows ? batch_sweep_occupancy_inst<Recover64, true>(threads, smem)
                : batch_sweep_occupancy_inst<Recover64, false>(threads, smem);
}

}  // namespace mhd
