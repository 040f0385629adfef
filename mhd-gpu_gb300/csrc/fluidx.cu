// fluidx.cu - launch table of the fluid sweep and the faithful-policy
// instantiation (kernel in fluidx_kernel.cuh).
#include "fluidx_kernel.cuh"

namespace mhd {

// default team shape by pencil length (the autotuner can override it,
// tuning.cu); the team covers n <= 32*WPP*CPL
PencilCfg fluidx_pick(int n)
{
    if (n <= 32)  return {1, 1, 8};
    if (n <= 64)  return {2, 1, 4};
    if (n <= 128) return {4, 1, 4};
    if (n == 256) return {8, 1, 1};   // register-blocked, 8 cells per thread
    if (n <= 256) return {4, 2, 2};
    if (n <= 512) return {4, 4, 1};
    return {4, 8, 1};
}

cudaError_t launch_fluidx_faithful(const FluidxArgs &a, const PencilCfg &cfg, cudaStream_t s)
{
    return launch_fluidx_policy<Faithful>(a, cfg, s);
}

// a frame the kernels can stage: contiguous pencils in the reference layout
// with identity component maps, or pencils across memory with sj == 1
bool frame_supported(const Frame &f)
{
    if (!frame_rows(f))
        return f.sj == f.n && f.sk == (long long)f.n * f.ny && f.pu == 0x43210u && f.pb == 0x210u;
    return f.sj == 1;
}

cudaError_t launch_fluidx(const FluidxArgs &a, const PencilCfg &cfg, int math, cudaStream_t s)
{
    if (!pencil_shape_ok(cfg, a.f.n) || !frame_supported(a.f)) return cudaErrorInvalidConfiguration;
    if (math == MHD_MATH_FAST) return launch_fluidx_fast(a, cfg, s);
    if (math == MHD_MATH_FP64P) return launch_fluidx_p64(a, cfg, s);
    return launch_fluidx_faithful(a, cfg, s);
}

}  // namespace mhd
