// compat.cu - host-pointer shims with the reference C path's names and
// signatures (Heterogeneous_MHD/C/spu_function.h:1-15), declared in
// include/mhdgpu_compat.h.  A driver written for the reference (mhd.c) links
// against these unchanged: each call uploads its inputs, runs the sm_103a
// kernel and downloads the result, synchronously, as the reference's calls
// return with the work done.  They exist for drop-in use and parity checks;
// the stream-ordered device API in include/mhdgpu.h is the fast path.
//
// Device buffers are cached per thread and grow on demand (the reference's
// own C path keeps static scratch the same way, C/fluidx.c:9-15).  Errors are
// reported on stderr and through mhdgpu_compat_status(); the reference
// functions return void, so there is no other channel.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>
#include <vector>

#include "mhdgpu.h"
#include "mhdgpu_compat.h"
#include "mhdgpu_fortran.h"

namespace {

struct CompatCtx {
    float *du = nullptr, *db = nullptr, *du2 = nullptr, *db2 = nullptr, *scr = nullptr, *dt = nullptr;
    unsigned *word = nullptr;
    size_t cap = 0;   // cells
    int status = MHD_OK;

    ~CompatCtx()
    {
        cudaFree(du); cudaFree(db); cudaFree(du2); cudaFree(db2); cudaFree(scr); cudaFree(dt); cudaFree(word);
    }

    bool ensure(size_t ncell)
    {
        if (ncell <= cap && du) return true;
        cudaFree(du); cudaFree(db); cudaFree(du2); cudaFree(db2); cudaFree(scr); cudaFree(dt); cudaFree(word);
        du = db = du2 = db2 = scr = dt = nullptr;
        word = nullptr;
        cap = 0;
        if (cudaMalloc(&du, ncell * 5 * sizeof(float)) != cudaSuccess) return false;
        if (cudaMalloc(&db, ncell * 3 * sizeof(float)) != cudaSuccess) return false;
        if (cudaMalloc(&du2, ncell * 5 * sizeof(float)) != cudaSuccess) return false;
        if (cudaMalloc(&db2, ncell * 3 * sizeof(float)) != cudaSuccess) return false;
        if (cudaMalloc(&scr, ncell * 2 * sizeof(float)) != cudaSuccess) return false;
        if (cudaMalloc(&dt, 4 * sizeof(float)) != cudaSuccess) return false;
        if (cudaMalloc(&word, sizeof(unsigned)) != cudaSuccess) return false;
        cap = ncell;
        return true;
    }
};

thread_local CompatCtx g_ctx;

bool report(int st, const char *who)
{
    g_ctx.status = st;
    if (st != MHD_OK) fprintf(stderr, "%s: %s (%s)\n", who, mhdgpu_status_string(st), mhdgpu_last_error());
    return st == MHD_OK;
}

bool cuda_ok(cudaError_t e, const char *who)
{
    if (e == cudaSuccess) return true;
    fprintf(stderr, "%s: %s\n", who, cudaGetErrorString(e));
    g_ctx.status = MHD_ERR_CUDA;
    return false;
}

size_t cells(const int *nx, const int *ny, const int *nz)
{
    return (size_t)(*nx) * (size_t)(*ny) * (size_t)(*nz);
}

}  // namespace

extern "C" {

int mhdgpu_compat_status(void) { return g_ctx.status; }

void fluidx(float *u, float *b, int *nx, int *ny, int *nz, float *dt, float *update_u,
            float *update_b, int iter)
{
    (void)b; (void)iter;
    const size_t nc = cells(nx, ny, nz);
    if (!g_ctx.ensure(nc)) { report(MHD_ERR_NOMEM, "fluidx"); return; }
    if (!cuda_ok(cudaMemcpy(g_ctx.du, update_u, nc * 5 * sizeof(float), cudaMemcpyHostToDevice), "fluidx")) return;
    if (!cuda_ok(cudaMemcpy(g_ctx.db, update_b, nc * 3 * sizeof(float), cudaMemcpyHostToDevice), "fluidx")) return;
    if (!cuda_ok(cudaMemcpy(g_ctx.dt, dt, sizeof(float), cudaMemcpyHostToDevice), "fluidx")) return;
    if (!report(mhdgpu_fluidx(g_ctx.du, g_ctx.du, g_ctx.db, *nx, *ny, *nz, g_ctx.dt, nullptr, nullptr), "fluidx")) return;
    cuda_ok(cudaMemcpy(u, g_ctx.du, nc * 5 * sizeof(float), cudaMemcpyDeviceToHost), "fluidx");
}

void advectbyzx(float *u, float *b, int *nx, int *ny, int *nz, float *dt, float *update_u,
                float *update_b)
{
    (void)u;
    const size_t nc = cells(nx, ny, nz);
    if (!g_ctx.ensure(nc)) { report(MHD_ERR_NOMEM, "advectbyzx"); return; }
    // the reference reads b_y, b_z from update_b and b_x from b (A1.c:67, B1.c:60, A1.c:79)
    std::vector<float> merged(update_b, update_b + nc * 3);
    for (size_t c = 0; c < nc; ++c) merged[c * 3] = b[c * 3];
    if (!cuda_ok(cudaMemcpy(g_ctx.du, update_u, nc * 5 * sizeof(float), cudaMemcpyHostToDevice), "advectbyzx")) return;
    if (!cuda_ok(cudaMemcpy(g_ctx.db, merged.data(), nc * 3 * sizeof(float), cudaMemcpyHostToDevice), "advectbyzx")) return;
    if (!cuda_ok(cudaMemcpy(g_ctx.dt, dt, sizeof(float), cudaMemcpyHostToDevice), "advectbyzx")) return;
    if (!report(mhdgpu_advectbyzx(g_ctx.db, g_ctx.du, *nx, *ny, *nz, g_ctx.dt, g_ctx.scr, nullptr), "advectbyzx")) return;
    cuda_ok(cudaMemcpy(b, g_ctx.db, nc * 3 * sizeof(float), cudaMemcpyDeviceToHost), "advectbyzx");
}

static void transpose_shim(float *u, float *b, float *update_u, float *update_b, int *nx, int *ny,
                           int *nz, int which, const char *who)
{
    const size_t nc = cells(nx, ny, nz);
    if (!g_ctx.ensure(nc)) { report(MHD_ERR_NOMEM, who); return; }
    if (!cuda_ok(cudaMemcpy(g_ctx.du, update_u, nc * 5 * sizeof(float), cudaMemcpyHostToDevice), who)) return;
    if (!cuda_ok(cudaMemcpy(g_ctx.db, update_b, nc * 3 * sizeof(float), cudaMemcpyHostToDevice), who)) return;
    int st = which == 12
                 ? mhdgpu_transpose12(g_ctx.du2, g_ctx.db2, g_ctx.du, g_ctx.db, *nx, *ny, *nz, nullptr)
                 : mhdgpu_transpose13(g_ctx.du2, g_ctx.db2, g_ctx.du, g_ctx.db, *nx, *ny, *nz, nullptr);
    if (!report(st, who)) return;
    if (!cuda_ok(cudaMemcpy(u, g_ctx.du2, nc * 5 * sizeof(float), cudaMemcpyDeviceToHost), who)) return;
    cuda_ok(cudaMemcpy(b, g_ctx.db2, nc * 3 * sizeof(float), cudaMemcpyDeviceToHost), who);
}

void transpose12(float *u, float *b, float *update_u, float *update_b, int *nx, int *ny, int *nz,
                 int iter)
{
    (void)iter;
    transpose_shim(u, b, update_u, update_b, nx, ny, nz, 12, "transpose12");
}

void transpose13(float *u, float *b, float *update_u, float *update_b, int *nx, int *ny, int *nz)
{
    transpose_shim(u, b, update_u, update_b, nx, ny, nz, 13, "transpose13");
}

float calcfl(float *u, float *b, int *nx, int *ny, int *nz)
{
    const size_t nc = cells(nx, ny, nz);
    float inv = 0.0f;
    if (!g_ctx.ensure(nc)) { report(MHD_ERR_NOMEM, "calcfl"); return inv; }
    if (!cuda_ok(cudaMemcpy(g_ctx.du, u, nc * 5 * sizeof(float), cudaMemcpyHostToDevice), "calcfl")) return inv;
    if (!cuda_ok(cudaMemcpy(g_ctx.db, b, nc * 3 * sizeof(float), cudaMemcpyHostToDevice), "calcfl")) return inv;
    if (!report(mhdgpu_cfl(g_ctx.du, g_ctx.db, *nx, *ny, *nz, MHD_CFL_C, g_ctx.dt, g_ctx.word, nullptr), "calcfl"))
        return inv;
    cuda_ok(cudaMemcpy(&inv, g_ctx.dt, sizeof(float), cudaMemcpyDeviceToHost), "calcfl");
    return inv;
}

void copy_matrix(float *u, float *b, int *nx, int *ny, int *nz, float *update_u, float *update_b)
{
    // host arrays in the reference's calling convention: a host copy
    const size_t nc = cells(nx, ny, nz);
    memcpy(update_u, u, nc * 5 * sizeof(float));
    memcpy(update_b, b, nc * 3 * sizeof(float));
}

// ---- Fortran ABI (include/mhdgpu_fortran.h): the external subroutines of
// OpenMP/mhd.f90:249-474 as gfortran names them (lower case, trailing
// underscore, every argument by reference), host arrays, synchronous.

void fluidx_(float *u, float *b, int *nx, int *ny, int *nz, float *dt)
{
    const size_t nc = cells(nx, ny, nz);
    if (!g_ctx.ensure(nc)) { report(MHD_ERR_NOMEM, "fluidx_"); return; }
    if (!cuda_ok(cudaMemcpy(g_ctx.du, u, nc * 5 * sizeof(float), cudaMemcpyHostToDevice), "fluidx_")) return;
    if (!cuda_ok(cudaMemcpy(g_ctx.db, b, nc * 3 * sizeof(float), cudaMemcpyHostToDevice), "fluidx_")) return;
    if (!cuda_ok(cudaMemcpy(g_ctx.dt, dt, sizeof(float), cudaMemcpyHostToDevice), "fluidx_")) return;
    if (!report(mhdgpu_fluidx(g_ctx.du, g_ctx.du, g_ctx.db, *nx, *ny, *nz, g_ctx.dt, nullptr, nullptr), "fluidx_")) return;
    cuda_ok(cudaMemcpy(u, g_ctx.du, nc * 5 * sizeof(float), cudaMemcpyDeviceToHost), "fluidx_");
}

void advectbyzx_(float *u, float *b, int *nx, int *ny, int *nz, float *dt)
{
    const size_t nc = cells(nx, ny, nz);
    if (!g_ctx.ensure(nc)) { report(MHD_ERR_NOMEM, "advectbyzx_"); return; }
    if (!cuda_ok(cudaMemcpy(g_ctx.du, u, nc * 5 * sizeof(float), cudaMemcpyHostToDevice), "advectbyzx_")) return;
    if (!cuda_ok(cudaMemcpy(g_ctx.db, b, nc * 3 * sizeof(float), cudaMemcpyHostToDevice), "advectbyzx_")) return;
    if (!cuda_ok(cudaMemcpy(g_ctx.dt, dt, sizeof(float), cudaMemcpyHostToDevice), "advectbyzx_")) return;
    if (!report(mhdgpu_advectbyzx(g_ctx.db, g_ctx.du, *nx, *ny, *nz, g_ctx.dt, g_ctx.scr, nullptr), "advectbyzx_"))
        return;
    cuda_ok(cudaMemcpy(b, g_ctx.db, nc * 3 * sizeof(float), cudaMemcpyDeviceToHost), "advectbyzx_");
}

// The Fortran driver transposes in place, transpose12(u,b,u,b,...): the
// shim reads the whole input before it writes the output, so ut may be u.
void transpose12_(float *ut, float *bt, float *u, float *b, int *nx, int *ny, int *nz)
{
    transpose_shim(ut, bt, u, b, nx, ny, nz, 12, "transpose12_");
}

void transpose13_(float *ut, float *bt, float *u, float *b, int *nx, int *ny, int *nz)
{
    transpose_shim(ut, bt, u, b, nx, ny, nz, 13, "transpose13_");
}

// The Fortran cfl (mhd.f90:96-125) is internal to the main program and sees
// the sizes by host association; as an external function it takes them.
// Release 0.2 formula (B averaged to the cell centre); returns 1/c.
float cfl_(float *u, float *b, int *nx, int *ny, int *nz)
{
    const size_t nc = cells(nx, ny, nz);
    float inv = 0.0f;
    if (!g_ctx.ensure(nc)) { report(MHD_ERR_NOMEM, "cfl_"); return inv; }
    if (!cuda_ok(cudaMemcpy(g_ctx.du, u, nc * 5 * sizeof(float), cudaMemcpyHostToDevice), "cfl_")) return inv;
    if (!cuda_ok(cudaMemcpy(g_ctx.db, b, nc * 3 * sizeof(float), cudaMemcpyHostToDevice), "cfl_")) return inv;
    if (!report(mhdgpu_cfl(g_ctx.du, g_ctx.db, *nx, *ny, *nz, MHD_CFL_AVERAGED, g_ctx.dt, g_ctx.word, nullptr), "cfl_"))
        return inv;
    cuda_ok(cudaMemcpy(&inv, g_ctx.dt, sizeof(float), cudaMemcpyDeviceToHost), "cfl_");
    return inv;
}

}  // extern "C"
