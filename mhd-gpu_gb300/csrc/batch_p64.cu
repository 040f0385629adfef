// batch_p64.cu - the batched class kernels under the faithful policy with
// FP64 pressure recovery in low-beta cells (batch_kernel.cuh).
#include "batch_kernel.cuh"

namespace mhd {

cudaError_t launch_batch_class_p64(const ClassWork &w, int cls, bool rows, int grid, int threads,
                                  size_t smem, cudaStream_t s)
{
    return launch_batch_class_policy<Recover64>(w, cls, rows, grid, threads, smem, s);
}

int batch_class_occupancy_p64(int cls, bool rows, int threads, size_t smem)
{
    return batch_class_occupancy_policy<Recover64>(cls, rows, threads, smem);
}

}  // namespace mhd
