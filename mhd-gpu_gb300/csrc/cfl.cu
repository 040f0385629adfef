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
#include "kernels.cuh"

namespace mhd {

__global__ void __launch_bounds__(256)
cfl_kernel(const float *__restrict__ u, const float *__restrict__ b, int nx, int ny, int nz,
           int mode, unsigned *__restrict__ cmax)
{
    __shared__ float red[8];
    const long long ncell = (long long)nx * ny * nz;
    float cl = 0.0f;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell;
         c += (long long)gridDim.x * blockDim.x) {
        float uu[5], bb[3];
#pragma unroll
        for (int ii = 0; ii < 5; ++ii) uu[ii] = __ldg(u + c * 5 + ii);
        float cs;
        if (mode == MHD_CFL_C) {
#pragma unroll
            for (int ii = 0; ii < 3; ++ii) bb[ii] = __ldg(b + c * 3 + ii);
            cs = cfl_speed_c(uu, bb);
        } else {
            const long long pen = c / nx;
            const int i = (int)(c - pen * nx);
            const int j = (int)(pen % ny), k = (int)(pen / ny);
            const int ip = (i + 1 == nx) ? 0 : i + 1;
            const int jp = (j + 1 == ny) ? 0 : j + 1;
            const int kp = (k + 1 == nz) ? 0 : k + 1;
            const long long cx = ((long long)k * ny + j) * nx + ip;
            const long long cy = ((long long)k * ny + jp) * nx + i;
            const long long cz = ((long long)kp * ny + j) * nx + i;
            bb[0] = fdiv(fadd(__ldg(b + c * 3 + 0), __ldg(b + cx * 3 + 0)), 2.0f);
            bb[1] = fdiv(fadd(__ldg(b + c * 3 + 1), __ldg(b + cy * 3 + 1)), 2.0f);
            bb[2] = fdiv(fadd(__ldg(b + c * 3 + 2), __ldg(b + cz * 3 + 2)), 2.0f);
            cs = cfl_speed_averaged(uu, bb);
        }
        cl = fmaxf(cl, cs);   // fmaxf drops NaN like the reference's strict '>' scan
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cl = fmaxf(cl, __shfl_xor_sync(0xffffffffu, cl, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = cl;
    __syncthreads();
    if (threadIdx.x == 0) {
        float r = red[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = fmaxf(r, red[w]);
        atomicMax(cmax, __float_as_uint(r));
    }
}

// 1/c exactly as the reference's `temp1 = 1.0/c` (double divide, rounded to
// float); the word is cleared for the next reduction.
__global__ void cfl_finish_kernel(unsigned *cmax, float *inv_c)
{
    const float c = __uint_as_float(*cmax);
    *inv_c = (float)(1.0 / (double)c);
    *cmax = 0u;
}

// dt = cfl*(1/c) in double rounded to float; clamp to (tf-t)/2; t += 2dt.
__device__ __forceinline__ float dt_rule(float inv_c, double cfl_number, float t, float tf)
{
    float dt = (float)(cfl_number * (double)inv_c);
    if (tf > 0.0f) {
        const float rest = fdiv(fsub(tf, t), 2.0f);
        if (dt > rest) dt = rest;
    }
    return dt;
}

__global__ void dt_update_kernel(const float *inv_c, double cfl_number, float tf, float *t, float *dt)
{
    const float d = dt_rule(*inv_c, cfl_number, *t, tf);
    *dt = d;
    *t = fadd(*t, 2.0f * d);
}

// One iteration of the driver's clock: 1/c from the reduction word, dt, t,
// iteration count, dt log.  With tf > 0, once t >= tf (after the first step)
// the step runs with dt = 0, which leaves the state unchanged bit for bit:
// the reference's do { } while (t < tf) exit, without a host round trip.
__global__ void clock_kernel(mhdgpu_clock *clk, double cfl_number, float tf, float *dt_log)
{
    const float c = __uint_as_float(clk->cmax);
    clk->cmax = 0u;
    const float inv = (float)(1.0 / (double)c);
    clk->inv_c = inv;
    if (tf > 0.0f && clk->iter > 0 && !(clk->t < tf)) {
        clk->dt = 0.0f;
        return;
    }
    const float d = dt_rule(inv, cfl_number, clk->t, tf);
    clk->dt = d;
    clk->t = fadd(clk->t, 2.0f * d);
    if (dt_log) dt_log[clk->iter] = d;
    clk->iter += 1;
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
