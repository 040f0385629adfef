// debug.cu - the record of the debug build's index checks (mhd_debug.cuh)
// and its C-ABI readers.  In the release build the readers report a build
// without checks.
#include <cuda_runtime.h>

#include "mhd_debug.cuh"
#include "mhdgpu.h"

#undef MHD_DBG_FILE
#define MHD_DBG_FILE 10

namespace mhd {
#if defined(MHD_DEBUG)
__device__ unsigned g_dbg_count;
__device__ unsigned g_dbg_site;
__device__ long long g_dbg_index, g_dbg_extent;

__device__ __noinline__ bool debug_fault(unsigned kind, unsigned file, unsigned line, long long index,
                                         long long extent)
{
    if (atomicAdd(&g_dbg_count, 1u) == 0) {
        g_dbg_site = (kind << 28) | ((file & 0xffu) << 20) | (line & 0xfffffu);
        g_dbg_index = index;
        g_dbg_extent = extent;
    }
    return false;
}
#endif
}  // namespace mhd

namespace mhd {
// checks one index against an extent (nothing is accessed through it)
__global__ void debug_selftest_kernel(long long index, long long extent, int *in_bounds)
{
    *in_bounds = MHD_IN(index, extent) ? 1 : 0;
}
}  // namespace mhd

extern "C" int mhdgpu_debug_selftest(long long index, long long extent, int *in_bounds)
{
    if (!in_bounds) return MHD_ERR_ARG;
    int *d = nullptr;
    if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) return MHD_ERR_CUDA;
    mhd::debug_selftest_kernel<<<1, 1>>>(index, extent, d);
    const bool ok = cudaGetLastError() == cudaSuccess &&
                    cudaMemcpy(in_bounds, d, sizeof(int), cudaMemcpyDeviceToHost) == cudaSuccess;
    cudaFree(d);
    return ok ? MHD_OK : MHD_ERR_CUDA;
}

extern "C" int mhdgpu_debug_build(void)
{
#if defined(MHD_DEBUG)
    return 1;
#else
    return 0;
#endif
}

extern "C" int mhdgpu_debug_faults(unsigned *count, unsigned *kind, unsigned *file, unsigned *line,
                                   long long *index, long long *extent)
{
    unsigned c = 0, site = 0;
    long long i = 0, n = 0;
#if defined(MHD_DEBUG)
    if (cudaDeviceSynchronize() != cudaSuccess) return MHD_ERR_CUDA;
    if (cudaMemcpyFromSymbol(&c, mhd::g_dbg_count, sizeof c) != cudaSuccess ||
        cudaMemcpyFromSymbol(&site, mhd::g_dbg_site, sizeof site) != cudaSuccess ||
        cudaMemcpyFromSymbol(&i, mhd::g_dbg_index, sizeof i) != cudaSuccess ||
        cudaMemcpyFromSymbol(&n, mhd::g_dbg_extent, sizeof n) != cudaSuccess)
        return MHD_ERR_CUDA;
    const unsigned zero = 0;
    if (cudaMemcpyToSymbol(mhd::g_dbg_count, &zero, sizeof zero) != cudaSuccess) return MHD_ERR_CUDA;
#endif
    if (count) *count = c;
    if (kind) *kind = site >> 28;
    if (file) *file = (site >> 20) & 0xffu;
    if (line) *line = site & 0xfffffu;
    if (index) *index = i;
    if (extent) *extent = n;
    return MHD_OK;
}
