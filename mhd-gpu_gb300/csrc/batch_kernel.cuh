// batch_kernel.cuh - the batched ensemble: many independent periodic boxes of
// uneven, non-cubic sizes advance together, each sweep one set of concurrent
// persistent launches.
//
// There is no counterpart in the reference (its drivers advance one box,
// Heterogeneous_MHD/C/mhd.c:59-125); each box follows exactly the fused
// transpose-free step of one box (the same tile functions, the same rounding),
// so a box advanced in a batch is bit-identical to the box advanced alone.
//
// Team classes.  A sweep's boxes are grouped by the team class of their pencil
// length along the sweep (the length is a compile-time constant for 32, 48,
// 64, 96 and 128 cells), and each group is one persistent launch of a kernel
// specialised for its class; the groups of a sweep run concurrently (parallel
// branches of the step's graph) and the next sweep starts when all are done.
// A kernel holds one class only because classes compiled into one kernel share
// its register allocation and spill registers that none of them needs alone.
//
// Work list of a group.  A sweep has three phases per box: fluid tiles
// (fluidx_tile), field tiles (advect_tile) and b(1) chunks (advect_b1_cell),
// in the order fluid, field, b(1) on the way out and field, b(1), fluid on the
// way back (mhd.c:72-119).  The launch's items are (slot, box, item) triples,
// numbered slot-major through a prefix table, and CTAs claim them in that order
// from one atomic counter (the next claim is issued while the current item
// runs).  A phase of a box needs the box's previous phase complete (the field
// update reads u at the j-1 and k-1 pencils; b(1) reads the fluxes of the j+1
// and k+1 pencils); a CTA that claims such an item waits on the box's
// completion counter of the previous slot.  Every item waited on was claimed
// earlier by a running CTA, and the earliest unfinished item never waits, so
// the launch always drains whatever the residency; the wait is bounded all the
// same (batch_wait).
#pragma once

#include "advect_kernel.cuh"
#include "cfl_kernel.cuh"
#include "fluidx_kernel.cuh"

#undef MHD_DBG_FILE
#define MHD_DBG_FILE 5

namespace mhd {

constexpr int kBatchMaxPencil = MHD_BATCH_MAX_PENCIL;
constexpr int kBatchClasses = 8;

struct BoxDesc {
    float *u, *b;          // the caller's state, reference layout
    float *scr;            // 2 floats per cell: the shifted fluxes sA, sB
    mhdgpu_clock *clk;     // the box's clock (dt, t, health, CFL word)
    int nx, ny, nz, pad;
};

// team class by pencil length (1 <= n <= kBatchMaxPencil):
//   0: 32 = 1 x 32 threads     1: 64 = 2 x 32      2: 96 = 3 x 32
//   3: 128 = 4 x 32            4: 48 = 3 x 16 (half-warp teams)
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
// threads per pencil of a class
__host__ __device__ inline int batch_class_tpp(int c)
{
    return c == 4 ? 16 : (c == 6 ? 64 : (c == 7 ? 128 : 32));
}
__host__ __device__ inline int batch_tpp(int n) { return batch_class_tpp(batch_class(n)); }
// cells per thread and warps per pencil of a class (MHD_BATCH_CLASSES)
__host__ __device__ inline int batch_class_cpl(int c)
{
    return (c == 2 || c == 4) ? 3 : (c == 0 ? 1 : (c == 3 ? 4 : 2));
}
__host__ __device__ inline int batch_class_wpp(int c)
{
    return c == 4 ? 0 : (c == 6 ? 2 : (c == 7 ? 4 : 1));
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

// one persistent launch: up to kGroupBoxes boxes of one class in one sweep.
// The boxes' arguments travel in the launch's parameter block (read through
// the constant cache, like a single-box kernel's arguments), not in global
// memory, so the tile code reloads them for free instead of holding them in
// registers.
constexpr int kGroupBoxes = 64;
struct ClassWork {
    FluidxArgs fa[kGroupBoxes];   // each box's fluid-sweep arguments (frame of the sweep)
    AdvectArgs aa[kGroupBoxes];   // field-sweep arguments
    const long long *start;   // 3*nb + 1 prefix sums of item counts, entry slot*nb + box
    const int *group;         // 3*nb: tiles per item (fluid, field) or cells per item (b(1))
    unsigned *claim;          // next item of this launch (zeroed by the clock kernel)
    unsigned *done;           // 3*nb items finished per (slot, box) (zeroed likewise)
    unsigned *abort;          // nonzero once a dependency wait gave up
    int nb, fluid_first;
    unsigned stall_extra;     // test hook: extra items box 0's second phase waits for
};

// an item covers about this many cells (several tiles of small pencils), so
// the claim and the completion count cost little against the item's work
constexpr int kItemCells = 2048;
constexpr int kB1ItemCells = 4096;
// cells of a b(1) item a thread gathers at once
constexpr int kB1Group = 4;

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

__device__ __forceinline__ void batch_b1(const AdvectArgs &a, long long c0, int cells)
{
    const unsigned ncell = (unsigned)(a.f.npen * a.f.n);
    const unsigned c1 = min((unsigned)c0 + (unsigned)cells, ncell);
    const unsigned st = blockDim.x;
    unsigned c = (unsigned)c0 + threadIdx.x;
    for (; c + (kB1Group - 1) * st < c1; c += kB1Group * st)
        advect_b1_cells<kB1Group>(a, c, st);   // kB1Group cells' loads in flight
    for (; c < c1; c += st) advect_b1_cell(a, c);
}

// One sweep of the boxes of one class.  At most 256 threads per CTA; MINB
// resident CTAs of 256 threads per SM bound the registers (65536 / (256 MINB)).
template <int CPL, int WPP, class M, bool ROWS, int NT, int MINB>
__global__ void __launch_bounds__(256, MINB)
batch_class_kernel(const __grid_constant__ ClassWork w)
{
    __shared__ int s_e, s_run;
    __shared__ long long s_local;
    // the launch's prefix table (items < 2^31), items' sizes and, per (slot,
    // box), whether this CTA has already seen the entry's dependency complete
    __shared__ unsigned s_start[3 * kGroupBoxes + 1];
    __shared__ int s_group[3 * kGroupBoxes];
    __shared__ unsigned char s_ok[3 * kGroupBoxes];
    const int ne = MHD_IN(w.nb, kGroupBoxes + 1) ? 3 * w.nb : 0;
    for (int x = threadIdx.x; x <= ne; x += blockDim.x) s_start[x] = (unsigned)w.start[x];
    for (int x = threadIdx.x; x < ne; x += blockDim.x) {
        s_group[x] = w.group[x];
        s_ok[x] = 0;
    }
    __syncthreads();
    const unsigned total = s_start[ne];
    // thread 0 claims the next item while the CTA works on the current one;
    // a CTA's claims increase, so its entry only moves forward
    unsigned it = 0;
    int ecur = 0;
    if (threadIdx.x == 0) it = atomicAdd(w.claim, 1u);
    for (;;) {
        if (threadIdx.x == 0) {
            int e = -1, run = 0;
            long long local = 0;
            if (it < total) {
                while (MHD_IN(ecur + 1, ne + 1) && s_start[ecur + 1] <= it) ++ecur;   // last entry with start <= it
                e = ecur;
                local = (long long)(it - s_start[e]);
                run = 1;
                if (e >= w.nb && !s_ok[e - w.nb]) {   // wait for the box's previous phase
                    const int prev = e - w.nb;
                    const unsigned need = (s_start[prev + 1] - s_start[prev]) +
                                          (prev == 0 ? w.stall_extra : 0u);
                    run = batch_wait(w.done + prev, need, w.abort, w.fa[e % w.nb].health);
                    if (run) s_ok[prev] = 1;   // complete for good: later items skip the wait
                }
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
            const int slot = e / w.nb, bx = e - slot * w.nb;
            const int ph = batch_phase(slot, w.fluid_first);
            const long long local = s_local;
            const int g = s_group[e];
            if (ph == kPhaseB1) {
                batch_b1(w.aa[bx], local * g, g);
            } else {
                const int ppc = blockDim.x / team_threads<WPP>();
                const long long t0 = local * g;
                const long long t1 = min(t0 + g, batch_tiles(w.fa[bx].f, ppc, ROWS));
                for (long long t = t0; t < t1; ++t) {
                    if (t > t0) __syncthreads();   // the previous tile's shared memory is consumed
                    if (ph == kPhaseFluid) fluidx_tile<CPL, WPP, M, ROWS, NT, false, true>(w.fa[bx], t);
                    else advect_tile<CPL, WPP, M, ROWS, NT, true>(w.aa[bx], t);
                }
            }
        }
        // every write of the item is issued; count it with release semantics
        __syncthreads();
        if (threadIdx.x == 0) red_release_add(w.done + e, 1u);
    }
}

// the classes: (class, cells per thread, warps per pencil, compile-time
// length, CTAs per SM the registers are bounded for; warps per pencil 0 is a
// half-warp team).  The full-team classes fit 64 registers without spilling;
// uncapped, the compiler spends up to 128.
#define MHD_BATCH_CLASSES(X)                                                           \
    X(0, 1, 1, 32, 4) X(1, 2, 1, 64, 4) X(2, 3, 1, 96, 4) X(3, 4, 1, 128, 4) X(4, 3, 0, 48, 4) \
    X(5, 2, 1, 0, 2) X(6, 2, 2, 0, 2) X(7, 2, 4, 0, 2)

template <class M, bool ROWS>
const void *batch_class_kernel_ptr(int cls)
{
    switch (cls) {
#define MHD_BK(C, CPL, WPP, NT, MINB) \
    case C: return (const void *)batch_class_kernel<CPL, WPP, M, ROWS, NT, MINB>;
        MHD_BATCH_CLASSES(MHD_BK)
#undef MHD_BK
    default: return nullptr;
    }
}

template <class M>
cudaError_t launch_batch_class_policy(const ClassWork &w, int cls, bool rows, int grid, int threads,
                                      size_t smem, cudaStream_t s)
{
    const void *fn = rows ? batch_class_kernel_ptr<M, true>(cls) : batch_class_kernel_ptr<M, false>(cls);
    if (!fn || smem > 227 * 1024) return cudaErrorInvalidConfiguration;
    void *args[] = {const_cast<ClassWork *>(&w)};
    return cudaLaunchKernel(fn, dim3(grid), dim3(threads), args, smem, s);
}

// resident CTAs per SM of a class kernel; also raises its dynamic shared
// memory limit to smem (the launch relies on it)
template <class M>
int batch_class_occupancy_policy(int cls, bool rows, int threads, size_t smem)
{
    const void *fn = rows ? batch_class_kernel_ptr<M, true>(cls) : batch_class_kernel_ptr<M, false>(cls);
    if (!fn) return 0;
    if (smem > 48 * 1024 &&
        cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess)
        return 0;
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, threads, smem) != cudaSuccess) return 0;
    return nb;
}

// per-policy entry points (batch_faithful.cu, batch_fast.cu, batch_p64.cu)
cudaError_t launch_batch_class_faithful(const ClassWork &w, int cls, bool rows, int grid, int threads,
                                        size_t smem, cudaStream_t s);
cudaError_t launch_batch_class_fast(const ClassWork &w, int cls, bool rows, int grid, int threads,
                                    size_t smem, cudaStream_t s);
cudaError_t launch_batch_class_p64(const ClassWork &w, int cls, bool rows, int grid, int threads,
                                   size_t smem, cudaStream_t s);
int batch_class_occupancy_faithful(int cls, bool rows, int threads, size_t smem);
int batch_class_occupancy_fast(int cls, bool rows, int threads, size_t smem);
int batch_class_occupancy_p64(int cls, bool rows, int threads, size_t smem);

}  // namespace mhd
