// advect.cu - launchers of the field-advection kernels (advect_kernel.cuh)
// and the b(1) gather.
#include "advect_kernel.cuh"

namespace mhd {

template <int CPL, int WPP, class M, bool ROWS, int NT>
__global__ void __launch_bounds__(256)
advect_flux_kernel(const __grid_constant__ AdvectArgs a)
{
    advect_tile<CPL, WPP, M, ROWS, NT>(a, blockIdx.x);
}

// one thread per stored cell (advect_b1_cell, advect_kernel.cuh)
__global__ void __launch_bounds__(256)
advect_b1_kernel(const AdvectArgs a, unsigned ncell)
{
    const unsigned c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    advect_b1_cell(a, c);
}

PencilCfg advect_pick(int n)
{
    if (n <= 32)  return {1, 1, 8};
    if (n <= 64)  return {2, 1, 4};
    if (n <= 128) return {4, 1, 4};
    if (n == 256) return {2, 4, 1};
    if (n <= 256) return {4, 2, 2};
    if (n <= 512) return {4, 4, 1};
    return {4, 8, 1};
}

template <int CPL, int WPP, class M, bool ROWS, int NT>
static cudaError_t launch_advect_inst(const AdvectArgs &a, int ppc, cudaStream_t s)
{
    static std::atomic<size_t> smem_set[kSmemCacheDevices];
    const int threads = 32 * WPP * ppc;
    const long long blocks = ROWS ? (long long)((a.f.ny + ppc - 1) / ppc) * a.f.nz
                                  : (a.f.npen + ppc - 1) / ppc;
    const size_t smem = sizeof(float) * (size_t)ax_tile_smem_floats(NT > 0 ? NT : a.f.n, ppc, CPL, WPP, ROWS);
    if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
    const cudaError_t e = ensure_dynamic_smem((const void *)advect_flux_kernel<CPL, WPP, M, ROWS, NT>, smem, smem_set);
    if (e != cudaSuccess) return e;
    advect_flux_kernel<CPL, WPP, M, ROWS, NT><<<(unsigned)blocks, threads, smem, s>>>(a);
    return cudaGetLastError();
}

template <int C, int W, class M>
static cudaError_t launch_advect_shape(const AdvectArgs &a, int ppc, bool rows, cudaStream_t s)
{
    constexpr int CAP = 32 * W * C;
    if (a.f.n == CAP)
        return rows ? launch_advect_inst<C, W, M, true, CAP>(a, ppc, s)
                    : launch_advect_inst<C, W, M, false, CAP>(a, ppc, s);
    return rows ? launch_advect_inst<C, W, M, true, 0>(a, ppc, s)
                : launch_advect_inst<C, W, M, false, 0>(a, ppc, s);
}

template <class M>
static cudaError_t launch_advect_policy(const AdvectArgs &a, const PencilCfg &cfg, cudaStream_t s)
{
    const bool rows = frame_rows(a.f);
#define MHD_AX(C, W) \
    if (cfg.cpl == C && cfg.wpp == W) return launch_advect_shape<C, W, M>(a, cfg.ppc, rows, s);
    MHD_PENCIL_SHAPES(MHD_AX)
#undef MHD_AX
    return cudaErrorInvalidConfiguration;
}

cudaError_t launch_advect(const AdvectArgs &a, const PencilCfg &cfg, int math, cudaStream_t s)
{
    if (!pencil_shape_ok(cfg, a.f.n) || !frame_supported(a.f)) return cudaErrorInvalidConfiguration;
    cudaError_t e = (math == MHD_MATH_FAST) ? launch_advect_policy<Fast>(a, cfg, s)
                                            : launch_advect_policy<Faithful>(a, cfg, s);
    if (e != cudaSuccess) return e;
    const long long ncell = a.f.npen * a.f.n;
    const long long nb = (ncell + 255) / 256;
    advect_b1_kernel<<<(unsigned)nb, 256, 0, s>>>(a, (unsigned)ncell);
    return cudaGetLastError();
}

}  // namespace mhd
