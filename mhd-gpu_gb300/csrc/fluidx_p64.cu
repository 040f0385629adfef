// fluidx_p64.cu - the fluid sweep under the faithful policy with FP64
// pressure recovery in low-beta cells (Recover64, mhd_math.cuh; kernel in
// fluidx_kernel.cuh).  Compiled separately so the policies build in parallel.
#include "fluidx_kernel.cuh"

namespace mhd {

cudaError_t launch_fluidx_p64(const FluidxArgs &a, const PencilCfg &cfg, cudaStream_t s)
{
    return launch_fluidx_policy<Recover64>(a, cfg, s);
}

}  // namespace mhd
