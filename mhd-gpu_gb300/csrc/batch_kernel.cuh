// batch_kernel.cuh - the batched ensemble: many independent periodic boxes of
// uneven, non-cubic sizes advance together, one persistent launch per sweep.
//
// There is no counterpart in the reference (its drivers advance one box,
// Heterogeneous_MHD/C/mhd.c:59-125); each box follows exactly the fused
// transpose-free step of one box (the same tile functions, the same rounding),
// so a box advanced in a batch is bit-identical to the box advanced alone.
//
// Work list.  A sweep (x, y, z, z, y, x) has three phases per box: fluid
// tiles (fluidx_tile), field tiles (advect_tile) and b(1) chunks
// (advect_b1_cell), in the order fluid, field, b(1) on the way out and field,
// b(1), fluid on the way back (mhd.c:72-119).  The launch's items are the
// (slot, box, tile) triples, numbered slot-major through a prefix table, and
// CTAs claim them in that order from one atomic counter.  A phase of a box
// needs the box's previous phase complete (the field update reads u at the
// j-1 and k-1 pencils; b(1) reads the fluxes of the j+1 and k+1 pencils); a
// CTA that claims such an item waits on the box's completion counter of the
// previous slot.  Every item waited on was claimed earlier by a running CTA,
// and the earliest unfinished item never waits, so the launch always drains
// whatever the residency; the wait is bounded all the same (batch_wait).
//
// Team classes.  One kernel serves every pencil length of a sweep: the team
// shape is picked per item from the box's pencil length, with the length a
// compile-time constant for the ensemble's sizes (32, 48, 64, 96, 128) and at
// most three cells per thread.  Each class's tile is a separate (not inlined)
// function: inlined together in one kernel the classes spill registers that
// each of them alone does not need, and the call costs once per tile.  The
// kernel runs at 80 registers (3 CTAs of 256 threads per SM), where the
// full-team classes do not spill.  The item arguments are staged in shared
// memory.
#pragma once

#include "advect_kernel.cuh"
#include "cfl_kernel.cuh"
#include "fluidx_kernel.cuh"

namespace mhd {

constexpr int kBatchMaxPencil = MHD_BATCH_MAX_PENCIL;

struct BoxDesc {
    float *u, *b;          // the caller's state, reference layout
    float *scr;            // 2 floats per cell: the shifted fluxes sA, sB
    mhdgpu_clock *clk;     // the box's clock (dt, t, health, CFL word)
    int nx, ny, nz, pad;
};

// team class by pencil length (1 <= n <= kBatchMaxPencil); the length is a
// compile-time constant for 32, 48, 64, 96 and 128 cells:
//   0: 32 = 1 x 32 threads     1: 64 = 2 x 32      2: 96 = 3 x 32
//   3: 128 = 2 x 64            4: 48 (2 x 32, 16 slots idle)
//   5: other n < 64 (2 x 32)   6: other n < 128 (2 x 64)   7: n <= 256 (2 x 128)
__host__ __device__ inline int batch_class(int n)
{
    switch (n) {
    case 32: return 0;
    case 64: return 1;
    case 96: return 2;
    case 128: return 3;
    case 48: return 4;
    default: return n < 64 ? 5 : (n < 128 ? 6 : 7);
    }
}
// threads per pencil of the class
__host__ __device__ inline int batch_tpp(int n)
{
    const int c = batch_class(n);
    return (c == 3 || c == 6) ? 64 : (c == 7 ? 128 : 32);
}

// items of a phase: tiles of ppc pencils (contiguous pencils are numbered
// linearly, pencils across memory by (j-block, k)), or chunks of cells
__host__ __device__ inline long long batch_tiles(const Frame &f, int ppc, bool rows)
{
    return rows ? (long long)((f.ny + ppc - 1) / ppc) * f.nz : (f.npen + ppc - 1) / ppc;
}
__host__ __device__ inline long long batch_chunks(long long ncell, int chunk)
{
    return (ncell + chunk - 1) / chunk;
}
// phase of slot s: fluid-first sweeps run F, A, B1; the others A, B1, F
enum { kPhaseFluid = 0, kPhaseField = 1, kPhaseB1 = 2 };
__host__ __device__ inline int batch_phase(int slot, int fluid_first)
{
    return fluid_first ? slot : (slot + 1) % 3;
}

struct SweepWork {
    const BoxDesc *box;
    const long long *start;   // 3*nbox + 1 prefix sums of item counts, entry slot*nbox + box
    const int *group;         // 3*nbox: tiles per item (fluid, field) or cells per item (b(1))
    unsigned *claim;          // next item of this launch (zeroed by the clock kernel)
    unsigned *done;           // 3*nbox items finished per (slot, box) (zeroed likewise)
    unsigned *abort;          // nonzero once a dependency wait gave up
    int nbox, axis, fluid_first;
};

// an item covers about this many cells (several tiles of small pencils), so
// the claim and the completion count cost little against the item's work
constexpr int kItemCells = 2048;
constexpr int kB1ItemCells = 4096;

__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned *p)
{
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];\n" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// count an item done: a release reduction (no round trip), ordered after the
// CTA's writes by the barrier that precedes it
__device__ __forceinline__ void red_release_add(unsigned *p, unsigned v)
{
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;\n" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
    return t;
}

// Thread 0 of a CTA: wait until *ctr >= target.  Gives up after about two
// seconds (or 2^24 polls), or at once when another wait has given up: it then
// sets *abort and the box's STALL health bit and returns false, and the
// caller skips the item (the launch still drains; the state is invalid).
__device__ inline bool batch_wait(const unsigned *ctr, unsigned target, unsigned *abort,
                                  unsigned *health)
{
    if (ld_acquire_gpu(ctr) >= target) return true;
    const unsigned long long t0 = global_ns();
    for (int it = 0; it < (1 << 24); ++it) {
        __nanosleep(128);
        if (ld_acquire_gpu(ctr) >= target) return true;
        if (*(volatile unsigned *)abort) break;
        if (global_ns() - t0 > 2000000000ull) break;
    }
    atomicOr(abort, 1u);
    atomicOr(health, MHD_HEALTH_STALL);
    return false;
}

template <int C, int W, class M, bool ROWS, int NT>
__device__ __noinline__ void batch_fluidx_class(const FluidxArgs &a, long long tile)
{
    fluidx_tile<C, W, M, ROWS, NT>(a, tile);
}

template <int C, int W, class M, bool ROWS, int NT>
__device__ __noinline__ void batch_advect_class(const AdvectArgs &a, long long tile)
{
    advect_tile<C, W, M, ROWS, NT>(a, tile);
}

template <class M, bool ROWS>
__device__ __forceinline__ void batch_fluidx(const FluidxArgs &a, long long tile)
{
    switch (batch_class(a.f.n)) {
    case 0: batch_fluidx_class<1, 1, M, ROWS, 32>(a, tile); break;
    case 1: batch_fluidx_class<2, 1, M, ROWS, 64>(a, tile); break;
    case 2: batch_fluidx_class<3, 1, M, ROWS, 96>(a, tile); break;
    case 3: batch_fluidx_class<2, 2, M, ROWS, 128>(a, tile); break;
    case 4: batch_fluidx_class<2, 1, M, ROWS, 48>(a, tile); break;
    case 5: batch_fluidx_class<2, 1, M, ROWS, 0>(a, tile); break;
    case 6: batch_fluidx_class<2, 2, M, ROWS, 0>(a, tile); break;
    default: batch_fluidx_class<2, 4, M, ROWS, 0>(a, tile); break;
    }
}

template <class M, bool ROWS>
__device__ __forceinline__ void batch_advect(const AdvectArgs &a, long long tile)
{
    switch (batch_class(a.f.n)) {
    case 0: batch_advect_class<1, 1, M, ROWS, 32>(a, tile); break;
    case 1: batch_advect_class<2, 1, M, ROWS, 64>(a, tile); break;
    case 2: batch_advect_class<3, 1, M, ROWS, 96>(a, tile); break;
    case 3: batch_advect_class<2, 2, M, ROWS, 128>(a, tile); break;
    case 4: batch_advect_class<2, 1, M, ROWS, 48>(a, tile); break;
    case 5: batch_advect_class<2, 1, M, ROWS, 0>(a, tile); break;
    case 6: batch_advect_class<2, 2, M, ROWS, 0>(a, tile); break;
    default: batch_advect_class<2, 4, M, ROWS, 0>(a, tile); break;
    }
}

__device__ __forceinline__ void batch_b1(const AdvectArgs &a, long long c0, int cells)
{
    const long long ncell = a.f.npen * a.f.n;
    const long long c1 = min(c0 + cells, ncell);
    for (long long c = c0 + threadIdx.x; c < c1; c += blockDim.x) advect_b1_cell(a.b, a.sA, a.sB, a.f, c);
}

// One sweep of every box.  At most 256 threads (8 pencils of one warp per
// CTA); 3 CTAs per SM bound the registers at 80.
template <class M, bool ROWS>
__global__ void __launch_bounds__(256, 3)
batch_sweep_kernel(SweepWork w)
{
    __shared__ int s_e, s_run;
    __shared__ long long s_local;
    __shared__ FluidxArgs s_fa;
    __shared__ AdvectArgs s_aa;
    const long long total = w.start[3 * w.nbox];
    // thread 0 claims the next item while the CTA works on the current one
    unsigned it = 0;
    if (threadIdx.x == 0) it = atomicAdd(w.claim, 1u);
    for (;;) {
        if (threadIdx.x == 0) {
            int e = -1, run = 0;
            long long local = 0;
            if ((long long)it < total) {
                int lo = 0, hi = 3 * w.nbox - 1;   // last entry with start <= it
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (w.start[mid] <= (long long)it) lo = mid;
                    else hi = mid - 1;
                }
                e = lo;
                local = (long long)it - w.start[e];
                run = 1;
                if (e >= w.nbox) {   // wait for the box's previous phase
                    const int prev = e - w.nbox;
                    const unsigned need = (unsigned)(w.start[prev + 1] - w.start[prev]);
                    run = batch_wait(w.done + prev, need, w.abort, &w.box[e % w.nbox].clk->health);
                }
                const BoxDesc d = w.box[e % w.nbox];
                const Frame f = make_view(w.axis, d.nx, d.ny, d.nz);
                s_fa = FluidxArgs{d.u, d.u, d.b, &d.clk->dt, &d.clk->health, f};
                s_aa = AdvectArgs{d.b, d.u, &d.clk->dt, d.scr, d.scr + f.npen * f.n, f};
                it = atomicAdd(w.claim, 1u);
            }
            s_e = e;
            s_run = run;
            s_local = local;
        }
        __syncthreads();
        const int e = s_e;
        if (e < 0) break;
        if (s_run) {
            const int ph = batch_phase(e / w.nbox, w.fluid_first);
            const long long local = s_local;
            const int g = w.group[e];
            if (ph == kPhaseB1) {
                batch_b1(s_aa, local * g, g);
            } else {
                const int ppc = blockDim.x / batch_tpp(s_fa.f.n);
                const long long t0 = local * g;
                const long long t1 = min(t0 + g, batch_tiles(s_fa.f, ppc, ROWS));
                for (long long t = t0; t < t1; ++t) {
                    if (t > t0) __syncthreads();   // the previous tile's shared memory is consumed
                    if (ph == kPhaseFluid) batch_fluidx<M, ROWS>(s_fa, t);
                    else batch_advect<M, ROWS>(s_aa, t);
                }
            }
        }
        // every write of the item is issued; count it with release semantics
        __syncthreads();
        if (threadIdx.x == 0) red_release_add(w.done + e, 1u);
    }
}

template <class M, bool ROWS>
cudaError_t launch_batch_sweep_inst(const SweepWork &w, int grid, int threads, size_t smem, cudaStream_t s)
{
    static size_t smem_set = 0;
    if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
    if (smem > 48 * 1024 && smem_set < smem) {
        cudaError_t e = cudaFuncSetAttribute(batch_sweep_kernel<M, ROWS>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        smem_set = smem;
    }
    batch_sweep_kernel<M, ROWS><<<grid, threads, smem, s>>>(w);
    return cudaGetLastError();
}

template <class M, bool ROWS>
int batch_sweep_occupancy_inst(int threads, size_t smem)
{
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(batch_sweep_kernel<M, ROWS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)smem) != cudaSuccess)
        return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, batch_sweep_kernel<M, ROWS>, threads, smem) !=
        cudaSuccess)
        return 0;
    return nb;
}

// per-policy launchers (batch_faithful.cu, batch_fast.cu, batch_p64.cu)
cudaError_t launch_batch_sweep_faithful(const SweepWork &w, bool rows, int grid, int threads, size_t smem,
                                        cudaStream_t s);
cudaError_t launch_batch_sweep_fast(const SweepWork &w, bool rows, int grid, int threads, size_t smem,
                                    cudaStream_t s);
int batch_sweep_occupancy_faithful(bool rows, int threads, size_t smem);
int batch_sweep_occupancy_fast(bool rows, int threads, size_t smem);
cudaError_t launch_batch_sweep_p64(const SweepWork &w, bool rows, int grid, int threads, size_t smem,
                                   cudaStream_t s);
int batch_sweep_occupancy_p64(bool rows, int threads, size_t smem);

}  // namespace mhd
