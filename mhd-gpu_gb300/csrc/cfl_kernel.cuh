// cfl_kernel.cuh - per-cell CFL fast speed and the block max-reduction, shared
// by the single-box CFL kernel (cfl.cu) and the batched one (batch.cu).
// Formulas: Heterogeneous_MHD/C/calcfl.c:13-65 (MHD_CFL_C, unaveraged B) and
// OpenMP/mhd.f90:96-125 (MHD_CFL_AVERAGED, B averaged to the cell centre).
#pragma once

#include "kernels.cuh"

#undef MHD_DBG_FILE
#define MHD_DBG_FILE 7

namespace mhd {

__device__ __forceinline__ float cfl_cell_speed(const float *__restrict__ u, const float *__restrict__ b,
                                                int nx, int ny, int nz, int mode, long long c)
{
    float uu[5], bb[3];
    if (!MHD_IN(c, (long long)nx * ny * nz)) return 0.0f;
#pragma unroll
    for (int ii = 0; ii < 5; ++ii) uu[ii] = __ldg(u + c * 5 + ii);
    if (mode == MHD_CFL_C) {
#pragma unroll
        for (int ii = 0; ii < 3; ++ii) bb[ii] = __ldg(b + c * 3 + ii);
        return cfl_speed_c(uu, bb);
    }
    const long long pen = c / nx;
    const int i = (int)(c - pen * nx);
    const int j = (int)(pen % ny), k = (int)(pen / ny);
    const int ip = (i + 1 == nx) ? 0 : i + 1;
    const int jp = (j + 1 == ny) ? 0 : j + 1;
    const int kp = (k + 1 == nz) ? 0 : k + 1;
    const long long cx = ((long long)k * ny + j) * nx + ip;
    const long long cy = ((long long)k * ny + jp) * nx + i;
    const long long cz = ((long long)kp * ny + j) * nx + i;
    const long long ncell = (long long)nx * ny * nz;
    (void)ncell;
    if (!(MHD_IN(cx, ncell) && MHD_IN(cy, ncell) && MHD_IN(cz, ncell))) return 0.0f;
    bb[0] = fdiv(fadd(__ldg(b + c * 3 + 0), __ldg(b + cx * 3 + 0)), 2.0f);
    bb[1] = fdiv(fadd(__ldg(b + c * 3 + 1), __ldg(b + cy * 3 + 1)), 2.0f);
    bb[2] = fdiv(fadd(__ldg(b + c * 3 + 2), __ldg(b + cz * 3 + 2)), 2.0f);
    return cfl_speed_averaged(uu, bb);
}

// dt = cfl*(1/c) in double rounded to float; clamp to (tf-t)/2 (C/mhd.c:63-64)
__device__ __forceinline__ float dt_rule(float inv_c, double cfl_number, float t, float tf)
{
    float dt = (float)(cfl_number * (double)inv_c);
    if (tf > 0.0f) {
        const float rest = fdiv(fsub(tf, t), 2.0f);
        if (dt > rest) dt = rest;
    }
    return dt;
}

// One iteration of the driver's clock: 1/c from the reduction word, dt, t,
// iteration count, dt log.  With tf > 0, once t >= tf (after the first step)
// the step runs with dt = 0, which leaves the state unchanged bit for bit:
// the reference's do { } while (t < tf) exit, without a host round trip.
__device__ __forceinline__ void clock_tick(mhdgpu_clock *clk, double cfl_number, float tf, float *dt_log)
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
    if (dt_log && MHD_IN(clk->iter, 1 << 30)) dt_log[clk->iter] = d;
    clk->iter += 1;
}

}  // namespace mhd
