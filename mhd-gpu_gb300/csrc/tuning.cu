// tuning.cu - tile-shape table, arithmetic policy and the autotuner.
//
// The pencil kernels take their team shape (cells per thread, warps per
// pencil, pencils per CTA) from a table keyed by kernel class and pencil
// length, one per host thread like the other settings.  The default is a fixed table (fluidx_pick,
// advect_pick); mhdgpu_autotune measures every compiled shape with CUDA events
// on a synthetic state of the caller's box and records the fastest.
#include <cuda_runtime.h>
#include <stdio.h>

#include <atomic>
#include <map>
#include <mutex>
#include <vector>

#include "kernels.cuh"
#include "tunecache.h"

namespace mhd {

static thread_local std::map<std::pair<int, int>, PencilCfg> g_tiles;
// per host thread: a setting made on one thread changes only that thread's launches
static thread_local int g_math = MHD_MATH_FAITHFUL;
static thread_local int g_staging = MHD_STAGING_CPASYNC;
static thread_local int g_poison = 0;

// Pencils across memory are staged in rows of PPC cells, so they want many
// pencils per CTA (a row of 8 cells is 160 bytes of u).  256-cell pencils take
// the register-blocked tile with 8 cells per thread (about 150 registers for
// the fluid update, so fewer pencils per CTA there).
PencilCfg rows_pick(int kclass, int n)
{
    if (n <= 32)  return {1, 1, 8};
    if (n <= 64)  return {2, 1, 8};
    if (n <= 128) return {4, 1, 8};
    if (n == 256) return kclass == MHD_KCLASS_FLUIDX ? PencilCfg{8, 1, 4} : PencilCfg{8, 1, 8};
    if (n <= 256) return {4, 2, 4};
    if (n <= 512) return {4, 4, 2};
    return {4, 8, 1};
}

static int tile_key(int kclass, bool rows) { return kclass | (rows ? MHD_TILE_ROWS : 0); }

PencilCfg pencil_cfg(int kclass, int n, bool rows)
{
    {
        auto it = g_tiles.find({tile_key(kclass, rows), n});
        if (it != g_tiles.end()) return it->second;
    }
    if (rows) return rows_pick(kclass, n);
    return kclass == MHD_KCLASS_ADVECT ? advect_pick(n) : fluidx_pick(n);
}

int math_mode() { return g_math; }
int row_staging() { return g_staging; }
bool poison_scratch() { return g_poison != 0; }

// synthetic state for timing: rho = 1 + small ripple, weak flow, B ~ (1, .1, .2)
__global__ void tune_fill_kernel(float *u, float *b, long long ncell)
{
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell;
         c += (long long)gridDim.x * blockDim.x) {
        const float s = 0.01f * (float)((c * 2654435761LL) & 1023) / 1023.0f;
        u[c * 5 + 0] = 1.0f + s;
        u[c * 5 + 1] = 0.05f - s;
        u[c * 5 + 2] = 0.02f + s;
        u[c * 5 + 3] = -0.03f;
        u[c * 5 + 4] = 2.1f;
        b[c * 3 + 0] = 1.0f;
        b[c * 3 + 1] = 0.1f + s;
        b[c * 3 + 2] = 0.2f;
    }
}

}  // namespace mhd

using namespace mhd;

extern "C" {

int mhdgpu_set_math(int mode)
{
    if (mode != MHD_MATH_FAITHFUL && mode != MHD_MATH_FAST && mode != MHD_MATH_FP64P) {
        set_last_error("mhdgpu_set_math: unknown mode");
        return -1;
    }
    const int prev = g_math;
    g_math = mode;
    return prev;
}

int mhdgpu_set_poison(int on)
{
    const int prev = g_poison;
    g_poison = on ? 1 : 0;
    return prev;
}

int mhdgpu_set_row_staging(int mode)
{
    if (mode != MHD_STAGING_TMA && mode != MHD_STAGING_CPASYNC) {
        set_last_error("mhdgpu_set_row_staging: unknown mode");
        return -1;
    }
    const int prev = g_staging;
    g_staging = mode;
    return prev;
}

static bool tile_class_ok(int kclass)
{
    const int base = kclass & ~MHD_TILE_ROWS;
    return base == MHD_KCLASS_FLUIDX || base == MHD_KCLASS_ADVECT;
}

int mhdgpu_set_tile(int kclass, int n, int cpl, int wpp, int ppc)
{
    if (!tile_class_ok(kclass)) {
        set_last_error("mhdgpu_set_tile: kclass must be MHD_KCLASS_FLUIDX or MHD_KCLASS_ADVECT "
                       "(optionally | MHD_TILE_ROWS)");
        return MHD_ERR_ARG;
    }
    PencilCfg c{cpl, wpp, ppc};
    if (n < 1 || n > MHD_MAX_PENCIL || !pencil_shape_ok(c, n)) {
        set_last_error("mhdgpu_set_tile: shape not compiled or does not cover the pencil");
        return MHD_ERR_ARG;
    }
    g_tiles[{kclass, n}] = c;
    return MHD_OK;
}

int mhdgpu_get_tile(int kclass, int n, int *cpl, int *wpp, int *ppc)
{
    if (!tile_class_ok(kclass) || n < 1 || n > MHD_MAX_PENCIL) {
        set_last_error("mhdgpu_get_tile: bad kernel class or pencil length");
        return MHD_ERR_ARG;
    }
    const PencilCfg c = pencil_cfg(kclass & ~MHD_TILE_ROWS, n, (kclass & MHD_TILE_ROWS) != 0);
    if (cpl) *cpl = c.cpl;
    if (wpp) *wpp = c.wpp;
    if (ppc) *ppc = c.ppc;
    return MHD_OK;
}

int mhdgpu_tile_cache_save(const char *path)
{
    if (!path) {
        set_last_error("mhdgpu_tile_cache_save: null path");
        return MHD_ERR_ARG;
    }
    const std::map<std::pair<int, int>, PencilCfg> tiles = g_tiles;
    FILE *f = fopen(path, "w");
    if (!f) {
        set_last_error("mhdgpu_tile_cache_save: cannot open the file");
        return MHD_ERR_ARG;
    }
    fprintf(f, "{\n  \"format\": \"mhdgpu tile cache 1\",\n  \"device\": \"%s\",\n  \"tiles\": [",
            tune_device_name().c_str());
    bool first = true;
    for (const auto &t : tiles) {
        fprintf(f, "%s\n    {\"kclass\": %d, \"n\": %d, \"cpl\": %d, \"wpp\": %d, \"ppc\": %d}",
                first ? "" : ",", t.first.first, t.first.second, t.second.cpl, t.second.wpp, t.second.ppc);
        first = false;
    }
    fprintf(f, "\n  ]\n}\n");
    const bool ok = fclose(f) == 0;
    if (!ok) {
        set_last_error("mhdgpu_tile_cache_save: write failed");
        return MHD_ERR_ARG;
    }
    return MHD_OK;
}

int mhdgpu_tile_cache_load(const char *path, int *applied)
{
    if (applied) *applied = 0;
    std::string text, dev;
    if (!path || !read_text(path, text)) {
        set_last_error("mhdgpu_tile_cache_load: cannot read the file");
        return MHD_ERR_ARG;
    }
    std::string fmt;
    if (!json_string(text, "format", fmt) || fmt != "mhdgpu tile cache 1" || !json_string(text, "device", dev)) {
        set_last_error("mhdgpu_tile_cache_load: not a tile cache");
        return MHD_ERR_ARG;
    }
    if (!same_device(dev, tune_device_name())) return MHD_OK;   // tuned on another device: nothing applies
    int count = 0;
    for (size_t p = text.find("{\"kclass\""); p != std::string::npos; p = text.find("{\"kclass\"", p + 1)) {
        int kc, n, cpl, wpp, ppc;
        if (sscanf(text.c_str() + p, " { \"kclass\" : %d , \"n\" : %d , \"cpl\" : %d , \"wpp\" : %d , \"ppc\" : %d }",
                   &kc, &n, &cpl, &wpp, &ppc) != 5) {
            set_last_error("mhdgpu_tile_cache_load: malformed entry");
            return MHD_ERR_ARG;
        }
        const int st = mhdgpu_set_tile(kc, n, cpl, wpp, ppc);
        if (st != MHD_OK) return st;
        ++count;
    }
    if (applied) *applied = count;
    return MHD_OK;
}

int mhdgpu_autotune(int nx, int ny, int nz, int math)
{
    if (nx < 1 || ny < 1 || nz < 1 || nx > MHD_MAX_PENCIL || ny > MHD_MAX_PENCIL || nz > MHD_MAX_PENCIL) {
        set_last_error("mhdgpu_autotune: bad box");
        return MHD_ERR_ARG;
    }
    if (math != MHD_MATH_FAITHFUL && math != MHD_MATH_FAST && math != MHD_MATH_FP64P) {
        set_last_error("mhdgpu_autotune: unknown math mode");
        return MHD_ERR_ARG;
    }
    const long long ncell = (long long)nx * ny * nz;
    float *u = nullptr, *u2 = nullptr, *b = nullptr, *scr = nullptr, *dt = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaStream_t s = nullptr;
    int ret = MHD_OK;
    auto cuda = [&](cudaError_t e, const char *what) {
        if (e != cudaSuccess && ret == MHD_OK) {
            char buf[256];
            snprintf(buf, sizeof buf, "mhdgpu_autotune: %s: %s", what, cudaGetErrorString(e));
            set_last_error(buf);
            ret = MHD_ERR_CUDA;
        }
        return ret == MHD_OK;
    };
    const float hdt = 0.01f;
    if (!cuda(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking), "stream")) return ret;
    if (cuda(cudaMalloc(&u, ncell * 5 * sizeof(float)), "alloc") &&
        cuda(cudaMalloc(&u2, ncell * 5 * sizeof(float)), "alloc") &&
        cuda(cudaMalloc(&b, ncell * 3 * sizeof(float)), "alloc") &&
        cuda(cudaMalloc(&scr, ncell * 2 * sizeof(float)), "alloc") &&
        cuda(cudaMalloc(&dt, sizeof(float)), "alloc") &&
        cuda(cudaMemcpyAsync(dt, &hdt, sizeof(float), cudaMemcpyHostToDevice, s), "upload") &&
        cuda(cudaEventCreate(&e0), "event") && cuda(cudaEventCreate(&e1), "event")) {
        tune_fill_kernel<<<1024, 256, 0, s>>>(u, b, ncell);
        cuda(cudaGetLastError(), "fill");
        const int lens[3] = {nx, ny, nz};
        const int other[3][2] = {{ny, nz}, {nx, nz}, {nx, ny}};
        // contiguous pencils: the transposed frames of the plain step (every
        // length); pencils across memory: the y and z views of the
        // transpose-free step
        for (int job = 0; job < 5 && ret == MHD_OK; ++job) {
            const bool rows = job >= 3;
            const int axis = rows ? job - 2 : job;
            const int n = lens[axis];
            bool seen = false;
            for (int a2 = rows ? 1 : 0; a2 < axis; ++a2) seen = seen || lens[a2] == n;
            if (seen) continue;
            const Frame f = rows ? make_view(axis, nx, ny, nz)
                                 : make_frame(n, other[axis][0], other[axis][1]);
            for (int kclass : {MHD_KCLASS_FLUIDX, MHD_KCLASS_ADVECT}) {
                float best = 1e30f;
                PencilCfg best_cfg = pencil_cfg(kclass, n, rows);
                std::vector<PencilCfg> cands;
#define MHD_CAND(C, W)                                                       \
                for (int ppc = 1; ppc <= 8; ppc *= 2) {                      \
                    PencilCfg c{C, W, ppc};                                  \
                    if (pencil_shape_ok(c, n) && 32 * W * C < 4 * n + 32 * W) cands.push_back(c); \
                }
                MHD_PENCIL_SHAPES(MHD_CAND)
#undef MHD_CAND
                for (const PencilCfg &c : cands) {
                    float ms_best = 1e30f;
                    for (int rep = 0; rep < 4 && ret == MHD_OK; ++rep) {
                        cuda(cudaEventRecord(e0, s), "record");
                        cudaError_t le;
                        if (kclass == MHD_KCLASS_FLUIDX) {
                            FluidxArgs a{u2, u, b, dt, nullptr, f};
                            le = launch_fluidx(a, c, math, s);
                        } else {
                            AdvectArgs a = make_advect_args(b, u, dt, scr, scr + ncell, f);
                            le = launch_advect(a, c, math, s);
                        }
                        if (le != cudaSuccess) { cudaGetLastError(); break; }   // shape not launchable here
                        cuda(cudaEventRecord(e1, s), "record");
                        cuda(cudaEventSynchronize(e1), "sync");
                        float ms = 0.0f;
                        cuda(cudaEventElapsedTime(&ms, e0, e1), "elapsed");
                        if (rep > 0 && ms < ms_best) ms_best = ms;   // rep 0 warms up
                    }
                    if (ms_best < best) { best = ms_best; best_cfg = c; }
                }
                if (ret == MHD_OK) g_tiles[{tile_key(kclass, rows), n}] = best_cfg;
            }
        }
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaFree(u); cudaFree(u2); cudaFree(b); cudaFree(scr); cudaFree(dt);
    cudaStreamSynchronize(s);
    cudaStreamDestroy(s);
    return ret;
}

}  // extern "C"
