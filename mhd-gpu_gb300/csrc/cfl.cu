// cfl.cu - CFL reduction and the on-device dt update, for sm_103a.
//
// Algorithm: Heterogeneous_MHD/C/calcfl.c:13-65 (mode MHD_CFL_C, unaveraged B)
// and OpenMP/mhd.f90:96-125 (mode MHD_CFL_AVERAGED, B averaged to the cell
// centre as Cuda/cuda_cfl.cu:101-124 does); dt from Heterogeneous_MHD/C/mhd.c:63-65.
//
// The reference CUDA path has every block write the same word (a race,
// Cuda/cuda_cfl.cu:137) and then reduces on the host with a device->host->
// device round trip of dt.  Here the maximum stays on the device: a
// grid-stride pass, a warp-shuffle max, one shared-memory step per block and
// one atomicMax per block on the float's bit pattern (monotone for
// non-negative floats), then a single-thread kernel turns c into 1/c and dt.
// The max is exact, so the order of the reduction does not matter.
#include "cfl_kernel.cuh"

namespace mhd {

__global__ void __launch_bounds__(256)
cfl_kernel(const float *__restrict__ u, const float *__restrict__ b, int nx, int ny, int nz,
           int mode, unsigned *__restrict__ cmax)
{
    const long long ncell = (long long)nx * ny * nz;
    float cl = 0.0f;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell;
         c += (long long)gridDim.x * blockDim.x)
        cl = fmaxf(cl, cfl_cell_speed(u, b, nx, ny, nz, mode, c));   // fmaxf drops NaN like the
                                                                     // reference's strict '>' scan
    cfl_block_max(cl, cmax);
}

// 1/c exactly as the reference's `temp1 = 1.0/c` (double divide, rounded to
// float); the word is cleared for the next reduction.
__global__ void cfl_finish_kernel(unsigned *cmax, float *inv_c)
{
    const float c = __uint_as_float(*cmax);
    *inv_c = (float)(1.0 / (double)c);
    *cmax = 0u;
}

__global__ void dt_update_kernel(const float *inv_c, double cfl_number, float tf, float *t, float *dt)
{
    const float d = dt_rule(*inv_c, cfl_number, *t, tf);
    *dt = d;
    *t = fadd(*t, 2.0f * d);
}

__global__ void clock_kernel(mhdgpu_clock *clk, double cfl_number, float tf, float *dt_log)
{
    clock_tick(clk, cfl_number, tf, dt_log);
}

int cfl_grid(long long ncell)
{
    long long g = (ncell + 255) / 256;
    const long long cap = 152LL * 8;   // a few waves of 256-thread blocks on 152 SMs
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

cudaError_t launch_cfl(const float *u, const float *b, int nx, int ny, int nz, int mode,
                       unsigned *cmax, cudaStream_t s)
{
    const long long ncell = (long long)nx * ny * nz;
    cfl_kernel<<<cfl_grid(ncell), 256, 0, s>>>(u, b, nx, ny, nz, mode, cmax);
    return cudaGetLastError();
}

cudaError_t launch_cfl_finish(unsigned *cmax, float *inv_c, cudaStream_t s)
{
    cfl_finish_kernel<<<1, 1, 0, s>>>(cmax, inv_c);
    return cudaGetLastError();
}

cudaError_t launch_dt_update(const float *inv_c, double cfl_number, float tf, float *t, float *dt,
                             cudaStream_t s)
{
    dt_update_kernel<<<1, 1, 0, s>>>(inv_c, cfl_number, tf, t, dt);
    return cudaGetLastError();
}

cudaError_t launch_clock(mhdgpu_clock *clk, double cfl_number, float tf, float *dt_log, cudaStream_t s)
{
    clock_kernel<<<1, 1, 0, s>>>(clk, cfl_number, tf, dt_log);
    return cudaGetLastError();
}

}  // namespace mhd
