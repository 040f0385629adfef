// kernels.cuh - argument blocks and launchers shared by the kernel files and
// the C ABI (capi.cu).  Private to the library.
#pragma once

#include <cuda_runtime.h>

#include <atomic>

#include "mhd_common.cuh"

namespace mhd {

struct FluidxArgs {
    float *u_out;
    const float *u_in;
    const float *b;
    const float *dt;
    unsigned *health;
    Frame f;
    // Optional, contiguous identity frames only (the last x sweep of a step):
    // fold the updated cells' CFL fast speed (mode MHD_CFL_C or
    // MHD_CFL_AVERAGED) into *cfl with atomicMax, which saves the next step's
    // reduction pass over the state.
    unsigned *cfl = nullptr;
    int cfl_mode = 0;
};

struct AdvectArgs {
    float *b;             // in place (b_y, b_z by the flux kernel, b_x by the gather)
    const float *u;
    const float *dt;
    float *sA;            // ncell: shifted stage-A flux
    float *sB;            // ncell: shifted stage-B flux
    Frame f;
    // the gather's index arithmetic: stored cell c -> frame j = (c / sj) % ny,
    // k = (c / sk) % nz, as multiplies (set by make_advect_args)
    FastDiv dsj, dny, dsk, dnz;
};

inline AdvectArgs make_advect_args(float *b, const float *u, const float *dt, float *sA, float *sB,
                                   const Frame &f)
{
    AdvectArgs a;
    a.b = b; a.u = u; a.dt = dt; a.sA = sA; a.sB = sB; a.f = f;
    a.dsj = make_fastdiv((unsigned)f.sj);
    a.dny = make_fastdiv((unsigned)f.ny);
    a.dsk = make_fastdiv((unsigned)f.sk);
    a.dnz = make_fastdiv((unsigned)f.nz);
    return a;
}

// team shape of the pencil kernels: CPL cells per thread, WPP warps per
// pencil, PPC pencils per CTA
struct PencilCfg { int cpl, wpp, ppc; };

// the (CPL, WPP) pairs that are compiled
#define MHD_PENCIL_SHAPES(X) \
    X(1, 1) X(2, 1) X(4, 1) X(8, 1) X(1, 2) X(2, 2) X(4, 2) X(1, 4) X(2, 4) X(4, 4) X(2, 8) X(4, 8)

inline bool pencil_shape_ok(const PencilCfg &c, int n)
{
    bool known = false;
#define MHD_SHAPE_KNOWN(C, W) known = known || (c.cpl == C && c.wpp == W);
    MHD_PENCIL_SHAPES(MHD_SHAPE_KNOWN)
#undef MHD_SHAPE_KNOWN
    return known && c.ppc >= 1 && 32 * c.wpp * c.ppc <= 256 && n <= 32 * c.wpp * c.cpl;
}

PencilCfg fluidx_pick(int n);
PencilCfg advect_pick(int n);
bool frame_supported(const Frame &f);
// the shape in use for a kernel class, pencil length and staging mode (rows:
// pencils across memory): the tuned one if the autotuner (or mhdgpu_set_tile)
// recorded it, else the default table
PencilCfg pencil_cfg(int kclass, int n, bool rows = false);
PencilCfg rows_pick(int kclass, int n);
int math_mode();
// how row-staged pencils are moved (MHD_STAGING_TMA or MHD_STAGING_CPASYNC;
// the calling host thread's setting)
int row_staging();
// whether the entries fill their scratch with NaN before use (the calling
// host thread's setting, mhdgpu_set_poison)
bool poison_scratch();
cudaError_t launch_fluidx(const FluidxArgs &a, const PencilCfg &cfg, int math, cudaStream_t s);
cudaError_t launch_fluidx_faithful(const FluidxArgs &a, const PencilCfg &cfg, cudaStream_t s);
cudaError_t launch_fluidx_fast(const FluidxArgs &a, const PencilCfg &cfg, cudaStream_t s);
cudaError_t launch_fluidx_p64(const FluidxArgs &a, const PencilCfg &cfg, cudaStream_t s);
cudaError_t launch_advect(const AdvectArgs &a, const PencilCfg &cfg, int math, cudaStream_t s);
cudaError_t launch_transpose(float *du, float *db, const float *su, const float *sb,
                             int nx, int ny, int nz, int which, cudaStream_t s);
cudaError_t launch_cfl(const float *u, const float *b, int nx, int ny, int nz, int mode,
                       unsigned *cmax, cudaStream_t s);
cudaError_t launch_cfl_finish(unsigned *cmax, float *inv_c, cudaStream_t s);
cudaError_t launch_dt_update(const float *inv_c, double cfl_number, float tf, float *t, float *dt,
                             cudaStream_t s);
cudaError_t launch_clock(mhdgpu_clock *clk, double cfl_number, float tf, float *dt_log,
                         cudaStream_t s);

// sets the calling thread's message returned by mhdgpu_last_error()
void set_last_error(const char *msg);
// drops mhdgpu_advectbyzx_noalloc's per-device scratch addresses (noalloc.cu)
void noalloc_forget_devices();

// Raises a kernel's dynamic shared-memory limit to smem when above the 48 KB
// default, once per device and size (cache: one word per device ordinal;
// devices beyond it set the attribute on every call).  Thread-safe.
constexpr int kSmemCacheDevices = 16;
inline cudaError_t ensure_dynamic_smem(const void *fn, size_t smem, std::atomic<size_t> *cache)
{
    if (smem <= 48 * 1024) return cudaSuccess;
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess) dev = -1;
    const bool cached = dev >= 0 && dev < kSmemCacheDevices;
    if (cached && cache[dev].load(std::memory_order_relaxed) >= smem) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess && cached) {
        size_t cur = cache[dev].load(std::memory_order_relaxed);
        while (cur < smem && !cache[dev].compare_exchange_weak(cur, smem)) {
        }
    }
    return e;
}

}  // namespace mhd
