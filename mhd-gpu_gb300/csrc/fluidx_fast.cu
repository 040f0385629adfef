// fluidx_fast.cu - fast-policy instantiation of the fluid sweep (plain FP32
// with FMA contraction and hardware reciprocal/root; kernel in
// fluidx_kernel.cuh).  Compiled separately so both policies build in parallel.
#include "fluidx_kernel.cuh"

namespace mhd {

cudaError_t launch_fluidx_fast(const FluidxArgs &a, const PencilCfg &cfg, cudaStream_t s)
{
    return launch_fluidx_policy<Fast>(a, cfg, s);
}

}  // namespace mhd
