// batch_faithful.cu - the batched sweep kernels under the faithful math
// policy (batch_kernel.cuh).
#include "batch_kernel.cuh"

namespace mhd {

cudaError_t launch_batch_sweep_faithful(const SweepWork &w, bool rows, int grid, int threads, size_t smem,
                                        cudaStream_t s)
{
    return rows ? launch_batch_sweep_inst<Faithful, true>(w, grid, threads, smem, s)
                : launch_batch_sweep_inst<Faithful, false>(w, grid, threads, smem, s);
}

int batch_sweep_occupancy_faithful(bool rows, int threads, size_t smem)
{
    return rows ? batch_sweep_occupancy_inst<Faithful, true>(threads, smem)
                : batch_sweep_occupancy_inst<Faithful, false>(threads, smem);
}

}  // namespace mhd
