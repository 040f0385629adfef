// capi.cu - the C ABI of include/mhdgpu.h: argument checks, status codes and
// the step driver that sequences the per-subroutine kernels.
//
// The step driver restates the reference's sweep order
// (Heterogeneous_MHD/C/mhd.c:72-119): x, then y after transpose12, z twice
// after transpose13, y after transpose13, x after transpose12, with the
// fluid/field order reversed on the way back.  The reference copies the whole
// state after every subroutine (copy_matrix, 16 per step); here fluidx and
// advectbyzx run in place and only the transposes move data, ping-ponging
// between the caller's state and the workspace.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include "kernels.cuh"
#include "profiler.cuh"

using namespace mhd;

static thread_local char g_err[512];

void mhd::set_last_error(const char *msg)
{
    snprintf(g_err, sizeof g_err, "%s", msg);
}

static int fail(int status, const char *fmt, const char *detail = nullptr)
{
    if (detail) snprintf(g_err, sizeof g_err, fmt, detail);
    else snprintf(g_err, sizeof g_err, "%s", fmt);
    return status;
}

static int cuda_fail(cudaError_t e, const char *where)
{
    snprintf(g_err, sizeof g_err, "%s: %s", where, cudaGetErrorString(e));
    return MHD_ERR_CUDA;
}

#define MHD_CU(call, where)                              \
    do {                                                 \
        cudaError_t e_ = (call);                         \
        if (e_ != cudaSuccess) return cuda_fail(e_, where); \
    } while (0)

static bool dims_ok(int nx, int ny, int nz)
{
    if (nx < 1 || ny < 1 || nz < 1) return false;
    if (nx > MHD_MAX_PENCIL) return false;
    const long long ncell = (long long)nx * ny * nz;
    return ncell <= (1LL << 31) / 8;   // 8 floats per cell addressable with int offsets
}

static int check_dims(int nx, int ny, int nz, const char *who)
{
    if (!dims_ok(nx, ny, nz)) {
        snprintf(g_err, sizeof g_err, "%s: bad box %dx%dx%d (each >= 1, nx <= %d, <= 2^28 cells)",
                 who, nx, ny, nz, MHD_MAX_PENCIL);
        return MHD_ERR_ARG;
    }
    return MHD_OK;
}

extern "C" {

const char *mhdgpu_status_string(int status)
{
    switch (status) {
    case MHD_OK: return "ok";
    case MHD_ERR_ARG: return "invalid argument";
    case MHD_ERR_CUDA: return "CUDA error";
    case MHD_ERR_TIMEOUT: return "device wait timed out";
    case MHD_ERR_UNPHYSICAL: return "unphysical state";
    case MHD_ERR_NOMEM: return "out of memory";
    default: return "unknown status";
    }
}

const char *mhdgpu_last_error(void) { return g_err; }

const char *mhdgpu_version(void) { return "mhdgpu 0.1 sm_103a"; }

int mhdgpu_fluidx(float *u_out, const float *u_in, const float *b, int nx, int ny, int nz,
                  const float *d_dt, unsigned *d_health, mhdgpu_stream_t stream)
{
    int st = check_dims(nx, ny, nz, "mhdgpu_fluidx");
    if (st) return st;
    if (!u_out || !u_in || !b || !d_dt) return fail(MHD_ERR_ARG, "mhdgpu_fluidx: null pointer");
    const long long n5 = 5LL * nx * ny * nz;
    if (u_out != u_in && u_out < u_in + n5 && u_in < u_out + n5)
        return fail(MHD_ERR_ARG, "mhdgpu_fluidx: u_out partially overlaps u_in");
    FluidxArgs a{u_out, u_in, b, d_dt, d_health, make_frame(nx, ny, nz)};
    ProfScope ps(MHD_KCLASS_FLUIDX, 1, (cudaStream_t)stream);
    MHD_CU(launch_fluidx(a, pencil_cfg(MHD_KCLASS_FLUIDX, nx), math_mode(), (cudaStream_t)stream), "mhdgpu_fluidx");
    return MHD_OK;
}

size_t mhdgpu_advectbyzx_scratch_bytes(int nx, int ny, int nz)
{
    if (!dims_ok(nx, ny, nz)) return 0;
    return sizeof(float) * 2 * (size_t)nx * ny * nz;
}

int mhdgpu_advectbyzx(float *b, const float *u, int nx, int ny, int nz, const float *d_dt,
                      float *d_scratch, mhdgpu_stream_t stream)
{
    int st = check_dims(nx, ny, nz, "mhdgpu_advectbyzx");
    if (st) return st;
    if (!b || !u || !d_dt || !d_scratch) return fail(MHD_ERR_ARG, "mhdgpu_advectbyzx: null pointer");
    const long long ncell = (long long)nx * ny * nz;
    if (poison_scratch())
        MHD_CU(cudaMemsetAsync(d_scratch, 0xFF, sizeof(float) * 2 * (size_t)ncell, (cudaStream_t)stream),
               "mhdgpu_advectbyzx poison");
    AdvectArgs a = make_advect_args(b, u, d_dt, d_scratch, d_scratch + ncell, make_frame(nx, ny, nz));
    ProfScope ps(MHD_KCLASS_ADVECT, 2, (cudaStream_t)stream);
    MHD_CU(launch_advect(a, pencil_cfg(MHD_KCLASS_ADVECT, nx), math_mode(), (cudaStream_t)stream), "mhdgpu_advectbyzx");
    return MHD_OK;
}

static int transpose_common(float *dst_u, float *dst_b, const float *src_u, const float *src_b,
                            int nx, int ny, int nz, int which, mhdgpu_stream_t stream)
{
    const char *who = which == 12 ? "mhdgpu_transpose12" : "mhdgpu_transpose13";
    if (nx < 1 || ny < 1 || nz < 1 || (long long)nx * ny * nz > (1LL << 28))
        return fail(MHD_ERR_ARG, "%s: bad box", who);
    if (!dst_u || !dst_b || !src_u || !src_b) return fail(MHD_ERR_ARG, "%s: null pointer", who);
    if (dst_u == src_u || dst_b == src_b) return fail(MHD_ERR_ARG, "%s: transposes are out of place", who);
    if ((which == 12 ? nz : ny) > 65535) return fail(MHD_ERR_ARG, "%s: outer extent above 65535", who);
    ProfScope ps(MHD_KCLASS_TRANSPOSE, 1, (cudaStream_t)stream);
    MHD_CU(launch_transpose(dst_u, dst_b, src_u, src_b, nx, ny, nz, which, (cudaStream_t)stream), who);
    return MHD_OK;
}

int mhdgpu_transpose12(float *dst_u, float *dst_b, const float *src_u, const float *src_b,
                       int nx, int ny, int nz, mhdgpu_stream_t stream)
{
    return transpose_common(dst_u, dst_b, src_u, src_b, nx, ny, nz, 12, stream);
}

int mhdgpu_transpose13(float *dst_u, float *dst_b, const float *src_u, const float *src_b,
                       int nx, int ny, int nz, mhdgpu_stream_t stream)
{
    return transpose_common(dst_u, dst_b, src_u, src_b, nx, ny, nz, 13, stream);
}

int mhdgpu_cfl(const float *u, const float *b, int nx, int ny, int nz, int mode, float *d_inv_c,
               unsigned *d_scratch, mhdgpu_stream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || (long long)nx * ny * nz > (1LL << 28))
        return fail(MHD_ERR_ARG, "mhdgpu_cfl: bad box");
    if (!u || !b || !d_inv_c || !d_scratch) return fail(MHD_ERR_ARG, "mhdgpu_cfl: null pointer");
    if (mode != MHD_CFL_C && mode != MHD_CFL_AVERAGED) return fail(MHD_ERR_ARG, "mhdgpu_cfl: bad mode");
    cudaStream_t s = (cudaStream_t)stream;
    MHD_CU(cudaMemsetAsync(d_scratch, 0, sizeof(unsigned), s), "mhdgpu_cfl");
    ProfScope ps(MHD_KCLASS_CFL, 2, s);
    MHD_CU(launch_cfl(u, b, nx, ny, nz, mode, d_scratch, s), "mhdgpu_cfl");
    MHD_CU(launch_cfl_finish(d_scratch, d_inv_c, s), "mhdgpu_cfl");
    return MHD_OK;
}

int mhdgpu_dt_update(const float *d_inv_c, double cfl_number, float tf, float *d_t, float *d_dt,
                     mhdgpu_stream_t stream)
{
    if (!d_inv_c || !d_t || !d_dt) return fail(MHD_ERR_ARG, "mhdgpu_dt_update: null pointer");
    if (!(cfl_number > 0.0)) return fail(MHD_ERR_ARG, "mhdgpu_dt_update: cfl_number must be > 0");
    MHD_CU(launch_dt_update(d_inv_c, cfl_number, tf, d_t, d_dt, (cudaStream_t)stream), "mhdgpu_dt_update");
    return MHD_OK;
}

int mhdgpu_copy_matrix(float *dst_u, float *dst_b, const float *src_u, const float *src_b,
                       int nx, int ny, int nz, mhdgpu_stream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1) return fail(MHD_ERR_ARG, "mhdgpu_copy_matrix: bad box");
    if (!dst_u || !dst_b || !src_u || !src_b) return fail(MHD_ERR_ARG, "mhdgpu_copy_matrix: null pointer");
    const size_t ncell = (size_t)nx * ny * nz;
    cudaStream_t s = (cudaStream_t)stream;
    MHD_CU(cudaMemcpyAsync(dst_u, src_u, ncell * 5 * sizeof(float), cudaMemcpyDeviceToDevice, s),
           "mhdgpu_copy_matrix");
    MHD_CU(cudaMemcpyAsync(dst_b, src_b, ncell * 3 * sizeof(float), cudaMemcpyDeviceToDevice, s),
           "mhdgpu_copy_matrix");
    return MHD_OK;
}

size_t mhdgpu_step_workspace_bytes(int nx, int ny, int nz)
{
    if (!dims_ok(nx, ny, nz) || ny > MHD_MAX_PENCIL || nz > MHD_MAX_PENCIL) return 0;
    return sizeof(float) * 10 * (size_t)nx * ny * nz;
}

// the last fluid sweep of a step, in place on the x-major state, optionally
// folding the next step's CFL reduction into it
static int fluidx_last(float *u, const float *b, int nx, int ny, int nz, const float *dt,
                       unsigned *health, unsigned *cfl, int cfl_mode, cudaStream_t s)
{
    if (!cfl) return mhdgpu_fluidx(u, u, b, nx, ny, nz, dt, health, (mhdgpu_stream_t)s);
    FluidxArgs a{u, u, b, dt, health, make_frame(nx, ny, nz), cfl, cfl_mode};
    ProfScope ps(MHD_KCLASS_FLUIDX, 1, s);
    MHD_CU(launch_fluidx(a, pencil_cfg(MHD_KCLASS_FLUIDX, nx), math_mode(), s), "step fluidx");
    return MHD_OK;
}

// one sweep pair in frame (n, a, c): fluid then field, or field then fluid
static int sweep(float *u, float *b, int n, int a, int c, const float *dt, float *scr,
                 unsigned *health, bool fluid_first, cudaStream_t s, unsigned *cfl = nullptr,
                 int cfl_mode = 0)
{
    int st;
    if (fluid_first) {
        if ((st = mhdgpu_fluidx(u, u, b, n, a, c, dt, health, (mhdgpu_stream_t)s))) return st;
        return mhdgpu_advectbyzx(b, u, n, a, c, dt, scr, (mhdgpu_stream_t)s);
    }
    if ((st = mhdgpu_advectbyzx(b, u, n, a, c, dt, scr, (mhdgpu_stream_t)s))) return st;
    return fluidx_last(u, b, n, a, c, dt, health, cfl, cfl_mode, s);
}

static int step_plain(float *u, float *b, int nx, int ny, int nz, const float *d_dt, void *d_work,
                      unsigned *d_health, cudaStream_t s, unsigned *cfl, int cfl_mode);
static int step_fused(float *u, float *b, int nx, int ny, int nz, const float *d_dt, void *d_work,
                      unsigned *d_health, cudaStream_t s, unsigned *cfl, int cfl_mode);

int mhdgpu_step(float *u, float *b, int nx, int ny, int nz, const float *d_dt, void *d_work,
                unsigned *d_health, mhdgpu_stream_t stream)
{
    return step_plain(u, b, nx, ny, nz, d_dt, d_work, d_health, (cudaStream_t)stream, nullptr, 0);
}

// the plain step; with cfl set, its last fluid sweep also folds the next
// step's CFL fast speeds into *cfl (mode cfl_mode)
static int step_plain(float *u, float *b, int nx, int ny, int nz, const float *d_dt, void *d_work,
                      unsigned *d_health, cudaStream_t s, unsigned *cfl, int cfl_mode)
{
    const mhdgpu_stream_t stream = (mhdgpu_stream_t)s;
    int st = check_dims(nx, ny, nz, "mhdgpu_step");
    if (st) return st;
    if (ny > MHD_MAX_PENCIL || nz > MHD_MAX_PENCIL)
        return fail(MHD_ERR_ARG, "mhdgpu_step: every axis becomes a pencil; each must be <= MHD_MAX_PENCIL");
    if (!u || !b || !d_dt || !d_work) return fail(MHD_ERR_ARG, "mhdgpu_step: null pointer");
    const size_t ncell = (size_t)nx * ny * nz;
    if (poison_scratch())
        MHD_CU(cudaMemsetAsync(d_work, 0xFF, mhdgpu_step_workspace_bytes(nx, ny, nz), s), "mhdgpu_step poison");
    float *u2 = (float *)d_work;
    float *b2 = u2 + 5 * ncell;
    float *scr = b2 + 3 * ncell;
    // x
    if ((st = sweep(u, b, nx, ny, nz, d_dt, scr, d_health, true, s))) return st;
    // y (frame ny, nx, nz)
    if ((st = mhdgpu_transpose12(u2, b2, u, b, nx, ny, nz, stream))) return st;
    if ((st = sweep(u2, b2, ny, nx, nz, d_dt, scr, d_health, true, s))) return st;
    // z twice (frame nz, nx, ny)
    if ((st = mhdgpu_transpose13(u, b, u2, b2, ny, nx, nz, stream))) return st;
    if ((st = sweep(u, b, nz, nx, ny, d_dt, scr, d_health, true, s))) return st;
    if ((st = sweep(u, b, nz, nx, ny, d_dt, scr, d_health, false, s))) return st;
    // y back (frame ny, nx, nz)
    if ((st = mhdgpu_transpose13(u2, b2, u, b, nz, nx, ny, stream))) return st;
    if ((st = sweep(u2, b2, ny, nx, nz, d_dt, scr, d_health, false, s))) return st;
    // x back
    if ((st = mhdgpu_transpose12(u, b, u2, b2, ny, nx, nz, stream))) return st;
    return sweep(u, b, nx, ny, nz, d_dt, scr, d_health, false, s, cfl, cfl_mode);
}

// one sweep pair on a frame view of the x-major state: fluid then field, or
// field then fluid; launches the kernels on the view directly
static int sweep_view(float *u, float *b, const Frame &f, const float *dt, float *scr,
                      unsigned *health, bool fluid_first, cudaStream_t s, unsigned *cfl = nullptr,
                      int cfl_mode = 0)
{
    const long long ncell = f.npen * f.n;
    FluidxArgs fa{u, u, b, dt, health, f, cfl, cfl_mode};
    AdvectArgs aa = make_advect_args(b, u, dt, scr, scr + ncell, f);
    for (int part = 0; part < 2; ++part) {
        if ((part == 0) == fluid_first) {
            ProfScope ps(MHD_KCLASS_FLUIDX, 1, s);
            MHD_CU(launch_fluidx(fa, pencil_cfg(MHD_KCLASS_FLUIDX, f.n, frame_rows(f)), math_mode(), s),
                   "fused fluidx");
        } else {
            ProfScope ps(MHD_KCLASS_ADVECT, 2, s);
            MHD_CU(launch_advect(aa, pencil_cfg(MHD_KCLASS_ADVECT, f.n, frame_rows(f)), math_mode(), s),
                   "fused advectbyzx");
        }
    }
    return MHD_OK;
}

size_t mhdgpu_step_fused_workspace_bytes(int nx, int ny, int nz)
{
    if (!dims_ok(nx, ny, nz) || ny > MHD_MAX_PENCIL || nz > MHD_MAX_PENCIL) return 0;
    return sizeof(float) * 2 * (size_t)nx * ny * nz;
}

int mhdgpu_step_fused(float *u, float *b, int nx, int ny, int nz, const float *d_dt, void *d_work,
                      unsigned *d_health, mhdgpu_stream_t stream)
{
    return step_fused(u, b, nx, ny, nz, d_dt, d_work, d_health, (cudaStream_t)stream, nullptr, 0);
}

static int step_fused(float *u, float *b, int nx, int ny, int nz, const float *d_dt, void *d_work,
                      unsigned *d_health, cudaStream_t s, unsigned *cfl, int cfl_mode)
{
    int st = check_dims(nx, ny, nz, "mhdgpu_step_fused");
    if (st) return st;
    if (ny > MHD_MAX_PENCIL || nz > MHD_MAX_PENCIL)
        return fail(MHD_ERR_ARG, "mhdgpu_step_fused: every axis becomes a pencil; each must be <= MHD_MAX_PENCIL");
    if (!u || !b || !d_dt || !d_work) return fail(MHD_ERR_ARG, "mhdgpu_step_fused: null pointer");
    float *scr = (float *)d_work;
    if (poison_scratch())
        MHD_CU(cudaMemsetAsync(d_work, 0xFF, mhdgpu_step_fused_workspace_bytes(nx, ny, nz), s),
               "mhdgpu_step_fused poison");
    const Frame fx = make_view(0, nx, ny, nz), fy = make_view(1, nx, ny, nz), fz = make_view(2, nx, ny, nz);
    if ((st = sweep_view(u, b, fx, d_dt, scr, d_health, true, s))) return st;
    if ((st = sweep_view(u, b, fy, d_dt, scr, d_health, true, s))) return st;
    if ((st = sweep_view(u, b, fz, d_dt, scr, d_health, true, s))) return st;
    if ((st = sweep_view(u, b, fz, d_dt, scr, d_health, false, s))) return st;
    if ((st = sweep_view(u, b, fy, d_dt, scr, d_health, false, s))) return st;
    return sweep_view(u, b, fx, d_dt, scr, d_health, false, s, cfl, cfl_mode);
}

int mhdgpu_resolve_path(int nx, int ny, int nz)
{
    return (ny <= 48 && nz <= 48) ? MHD_PATH_FUSED : MHD_PATH_PLAIN;
}

size_t mhdgpu_path_workspace_bytes(int nx, int ny, int nz, int path)
{
    if (path == MHD_PATH_AUTO) path = mhdgpu_resolve_path(nx, ny, nz);
    if (path == MHD_PATH_FUSED) return mhdgpu_step_fused_workspace_bytes(nx, ny, nz);
    if (path == MHD_PATH_PLAIN) return mhdgpu_step_workspace_bytes(nx, ny, nz);
    return 0;
}

int mhdgpu_advance(float *u, float *b, int nx, int ny, int nz, int nsteps, double cfl_number,
                   int cfl_mode, float tf, mhdgpu_clock *d_clock, float *d_dt_log, void *d_work,
                   int path, mhdgpu_stream_t stream)
{
    if (nsteps < 0) return fail(MHD_ERR_ARG, "mhdgpu_advance: nsteps < 0");
    if (!d_clock) return fail(MHD_ERR_ARG, "mhdgpu_advance: null clock");
    const bool resume = (cfl_mode & MHD_ADVANCE_RESUME) != 0;
    cfl_mode &= ~MHD_ADVANCE_RESUME;
    if (!(cfl_number > 0.0)) return fail(MHD_ERR_ARG, "mhdgpu_advance: cfl_number must be > 0");
    if (cfl_mode != MHD_CFL_C && cfl_mode != MHD_CFL_AVERAGED)
        return fail(MHD_ERR_ARG, "mhdgpu_advance: bad cfl mode");
    if (path == MHD_PATH_AUTO) path = mhdgpu_resolve_path(nx, ny, nz);
    if (path != MHD_PATH_PLAIN && path != MHD_PATH_FUSED)
        return fail(MHD_ERR_ARG, "mhdgpu_advance: bad path");
    // Every check of the step runs here, before the first launch: a call that
    // is rejected queues nothing and leaves the clock as it was.
    int st0 = check_dims(nx, ny, nz, "mhdgpu_advance");
    if (st0) return st0;
    if (ny > MHD_MAX_PENCIL || nz > MHD_MAX_PENCIL)
        return fail(MHD_ERR_ARG, "mhdgpu_advance: every axis becomes a pencil; each must be <= MHD_MAX_PENCIL");
    if (!u || !b || !d_work) return fail(MHD_ERR_ARG, "mhdgpu_advance: null state or workspace pointer");
    cudaStream_t s = (cudaStream_t)stream;
    // The CFL reduction runs as its own pass before the first step of the
    // call (unless the caller resumes); every step's last fluid sweep folds
    // the next step's reduction into the clock's word.  The pass clears the
    // word first: the state may have changed since a previous call's fold.
    for (int it = 0; it < nsteps; ++it) {
        const bool pass = it == 0 && !resume;
        {
            ProfScope ps(MHD_KCLASS_CFL, pass ? 2 : 1, s);
            if (pass) {
                MHD_CU(cudaMemsetAsync(&d_clock->cmax, 0, sizeof(unsigned), s), "mhdgpu_advance");
                MHD_CU(launch_cfl(u, b, nx, ny, nz, cfl_mode, &d_clock->cmax, s), "mhdgpu_advance");
            }
            MHD_CU(launch_clock(d_clock, cfl_number, tf, d_dt_log, s), "mhdgpu_advance");
        }
        int st = (path == MHD_PATH_FUSED)
                     ? step_fused(u, b, nx, ny, nz, &d_clock->dt, d_work, &d_clock->health, s, &d_clock->cmax,
                                  cfl_mode)
                     : step_plain(u, b, nx, ny, nz, &d_clock->dt, d_work, &d_clock->health, s, &d_clock->cmax,
                                  cfl_mode);
        if (st) return st;
    }
    return MHD_OK;
}

// The host-buffer entry's device memory and stream, kept per host thread
// between calls (allocating and mapping ~40 B/cell per call cost about a
// third of a 128^3 call); grown to the largest request, released by
// mhdgpu_release_host_cache or when the thread ends.
struct HostEntryCache {
    int device = -1;
    cudaStream_t s = nullptr;
    char *buf = nullptr;
    size_t cap = 0;
    void release()
    {
        if (s) cudaStreamSynchronize(s);
        if (buf) cudaFree(buf);
        if (s) cudaStreamDestroy(s);
        buf = nullptr;
        cap = 0;
        s = nullptr;
        device = -1;
    }
    ~HostEntryCache() { release(); }
};
static thread_local HostEntryCache g_host_cache;

static size_t align256(size_t n) { return (n + 255) & ~(size_t)255; }

int mhdgpu_run_host(float *u, float *b, int nx, int ny, int nz, double cfl_number, int cfl_mode,
                    float *t, float tf, int max_steps, float *dt_log, int *steps_done, int path)
{
    int st = check_dims(nx, ny, nz, "mhdgpu_run_host");
    if (st) return st;
    if (!u || !b || !t) return fail(MHD_ERR_ARG, "mhdgpu_run_host: null pointer");
    if (max_steps < 0) return fail(MHD_ERR_ARG, "mhdgpu_run_host: max_steps < 0");
    if (path == MHD_PATH_AUTO) path = mhdgpu_resolve_path(nx, ny, nz);
    if (path != MHD_PATH_PLAIN && path != MHD_PATH_FUSED)
        return fail(MHD_ERR_ARG, "mhdgpu_run_host: bad path");
    const size_t ncell = (size_t)nx * ny * nz;
    const size_t wbytes = path == MHD_PATH_FUSED ? mhdgpu_step_fused_workspace_bytes(nx, ny, nz)
                                                 : mhdgpu_step_workspace_bytes(nx, ny, nz);
    if (!wbytes) return fail(MHD_ERR_ARG, "mhdgpu_run_host: box too large for the step");
    // carve u, b, workspace, clock and dt log out of the thread's buffer
    const size_t o_b = align256(ncell * 5 * sizeof(float));
    const size_t o_w = o_b + align256(ncell * 3 * sizeof(float));
    const size_t o_c = o_w + align256(wbytes);
    const size_t o_l = o_c + align256(sizeof(mhdgpu_clock));
    const size_t need = o_l + align256(sizeof(float) * (max_steps > 0 ? max_steps : 1));
    HostEntryCache &hc = g_host_cache;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "mhdgpu_run_host: device");
    if (hc.device != dev) {
        hc.release();
        if ((e = cudaStreamCreateWithFlags(&hc.s, cudaStreamNonBlocking)) != cudaSuccess) {
            hc.s = nullptr;
            return cuda_fail(e, "mhdgpu_run_host: stream");
        }
        hc.device = dev;
    }
    if (hc.cap < need) {
        if (hc.buf) cudaFree(hc.buf);
        hc.buf = nullptr;
        hc.cap = 0;
        if ((e = cudaMalloc((void **)&hc.buf, need)) != cudaSuccess) {
            hc.buf = nullptr;
            return cuda_fail(e, "mhdgpu_run_host: alloc");
        }
        hc.cap = need;
    }
    cudaStream_t s = hc.s;
    float *du = (float *)hc.buf, *db = (float *)(hc.buf + o_b), *dlog = (float *)(hc.buf + o_l);
    void *dw = hc.buf + o_w;
    mhdgpu_clock *dclk = (mhdgpu_clock *)(hc.buf + o_c);
    int ret = MHD_OK;
#define RH(call, where) do { e = (call); if (e != cudaSuccess) { ret = cuda_fail(e, where); goto done; } } while (0)
    {
        mhdgpu_clock h;
        memset(&h, 0, sizeof h);
        h.t = *t;
        RH(cudaMemcpyAsync(dclk, &h, sizeof h, cudaMemcpyHostToDevice, s), "mhdgpu_run_host: upload");
        RH(cudaMemcpyAsync(du, u, ncell * 5 * sizeof(float), cudaMemcpyHostToDevice, s), "mhdgpu_run_host: upload");
        RH(cudaMemcpyAsync(db, b, ncell * 3 * sizeof(float), cudaMemcpyHostToDevice, s), "mhdgpu_run_host: upload");
        ret = mhdgpu_advance(du, db, nx, ny, nz, max_steps, cfl_number, cfl_mode, tf, dclk, dlog, dw,
                             path, (mhdgpu_stream_t)s);
        if (ret) goto done;
        RH(cudaMemcpyAsync(u, du, ncell * 5 * sizeof(float), cudaMemcpyDeviceToHost, s), "mhdgpu_run_host: download");
        RH(cudaMemcpyAsync(b, db, ncell * 3 * sizeof(float), cudaMemcpyDeviceToHost, s), "mhdgpu_run_host: download");
        RH(cudaMemcpyAsync(&h, dclk, sizeof h, cudaMemcpyDeviceToHost, s), "mhdgpu_run_host: download");
        RH(cudaStreamSynchronize(s), "mhdgpu_run_host: sync");
        if (dt_log && h.iter > 0)
            RH(cudaMemcpy(dt_log, dlog, sizeof(float) * h.iter, cudaMemcpyDeviceToHost), "mhdgpu_run_host: dt log");
        *t = h.t;
        if (steps_done) *steps_done = h.iter;
        if (h.health & (MHD_HEALTH_NONFINITE | MHD_HEALTH_DENSITY))
            ret = fail(MHD_ERR_UNPHYSICAL, "mhdgpu_run_host: health word reports NaN/Inf or rho <= 0");
    }
done:
    // nothing of this call may still run on the stream when it returns
    if (ret != MHD_OK) cudaStreamSynchronize(s);
#undef RH
    return ret;
}

int mhdgpu_release_host_cache(void)
{
    g_host_cache.release();
    noalloc_forget_devices();
    return MHD_OK;
}

}  // extern "C"
