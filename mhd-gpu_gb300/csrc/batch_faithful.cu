// batch_faithful.cu - the batched class kernels under the faithful policy (batch_kernel.cuh).
#include "batch_kernel.cuh"

namespace mhd {

cudaError_t launch_batch_class_faithful(const ClassWork &w, int cls, bool rows, int grid, int threads,
                                  size_t smem, cudaStream_t s)
{
    return launch_batch_class_policy<Faithful>(w, cls, rows, grid, threads, smem, s);
}

int batch_class_occupancy_faithful(int cls, bool rows, int threads, size_t smem)
{
    return batch_class_occupancy_policy<Faithful>(cls, rows, threads, smem);
}

}  // namespace mhd
