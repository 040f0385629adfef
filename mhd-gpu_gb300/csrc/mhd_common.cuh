// mhd_common.cuh - shared device plumbing for the sm_103a MHD kernels:
// pencil geometry, the pencil-team (one or more warps that own one pencil),
// neighbour exchange through shared memory, pencil-wide max reduction and the
// device health word.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mhd_debug.cuh"
#include "mhd_math.cuh"
#include "mhdgpu.h"   // include/ is on the include path (build.py)

#undef MHD_DBG_FILE
#define MHD_DBG_FILE 9

namespace mhd {

// Pencil geometry of one frame: the frame's axes (i, j, k) have extents
// (n, ny, nz) and cell strides (si, sj, sk) in the stored array, and frame
// component f of u (of b) is stored component (pu >> 4f) & 15 ((pb >> 4f) & 15);
// iu, ib are the inverse maps.  The reference layout u(5,n,ny,nz) seen as
// itself is si = 1, sj = n, sk = n*ny with identity maps (make_frame); the
// y and z sweeps of a box stored x-major are strided views of the same array
// (make_view), which is how the transpose-free step avoids transposing.
struct Frame {
    int n, ny, nz;
    long long npen;
    long long si, sj, sk;
    unsigned pu, pb, iu, ib;
};

__host__ __device__ inline Frame make_frame(int n, int ny, int nz)
{
    Frame f;
    f.n = n; f.ny = ny; f.nz = nz;
    f.npen = (long long)ny * (long long)nz;
    f.si = 1; f.sj = n; f.sk = (long long)n * ny;
    f.pu = 0x43210u; f.pb = 0x210u; f.iu = 0x43210u; f.ib = 0x210u;
    return f;
}

// Frames of the sweeps of an nx*ny*nz box stored x-major (axis 0, 1, 2 = x, y, z):
//   x: (x, y, z), u (rho, m_x, m_y, m_z, E), b (b_x, b_y, b_z)
//   y: (y, x, z), u (rho, m_y, m_x, m_z, E), b (b_y, b_x, b_z)   [after transpose12]
//   z: (z, x, y), u (rho, m_z, m_x, m_y, E), b (b_z, b_x, b_y)   [after transpose12, 13]
// (Heterogeneous_MHD/C/mhd.c:72-119 with transpose12.c / transpose13.c).
__host__ __device__ inline Frame make_view(int axis, int nx, int ny, int nz)
{
    Frame f;
    const long long sxy = (long long)nx * ny;
    if (axis == 0) return make_frame(nx, ny, nz);
    if (axis == 1) {
        f.n = ny; f.ny = nx; f.nz = nz;
        f.si = nx; f.sj = 1; f.sk = sxy;
        f.pu = 0x43120u; f.pb = 0x201u; f.iu = 0x43120u; f.ib = 0x201u;
    } else {
        f.n = nz; f.ny = nx; f.nz = ny;
        f.si = sxy; f.sj = 1; f.sk = nx;
        f.pu = 0x42130u; f.pb = 0x102u; f.iu = 0x41320u; f.ib = 0x021u;
    }
    f.npen = (long long)f.ny * f.nz;
    return f;
}

__host__ __device__ __forceinline__ int nib(unsigned m, int f) { return (int)((m >> (4 * f)) & 15u); }

// Staging mode of a frame: contiguous pencils (the reference layout seen as
// itself: si = 1 and identity component maps) or rows (any other view; its
// pencils run across memory with sj = 1).  A y or z view of a box with
// nx = 1 has si = 1 too, but permuted components: it is staged in rows.
__host__ __device__ inline bool frame_rows(const Frame &f)
{
    return !(f.si == 1 && f.pu == 0x43210u && f.pb == 0x210u);
}

// threads of a pencil team: WPP warps, or half a warp for WPP = 0
template <int WPP>
__host__ __device__ constexpr int team_threads() { return WPP == 0 ? 16 : 32 * WPP; }
__host__ __device__ constexpr int team_threads_of(int wpp) { return wpp == 0 ? 16 : 32 * wpp; }

// A pencil whose length fills a team of at most one warp exactly takes the
// register-blocked tiles (fluidx_reg.cuh, advect_reg.cuh): thread t owns the
// consecutive cells t*CPL .. t*CPL+CPL-1 and stencil neighbours come from the
// adjacent lanes by warp shuffle.  Host and device agree through this test.
__host__ __device__ constexpr bool reg_tile_shape(int n, int cpl, int wpp)
{
    return wpp <= 1 && n == team_threads_of(wpp) * cpl;
}

// Unsigned division of a cell index n < 2^31 by a fixed divisor d >= 1 as a
// multiply and a shift: with l = ceil(log2 d), s = 31 + l and m = ceil(2^s / d)
// (< 2^32), floor(n m / 2^s) = floor(n / d) for every n < 2^31, since
// m/2^s - 1/d < 2^-(31+l) and so n m / 2^s < n/d + 1/d (Granlund and
// Montgomery, "Division by invariant integers using multiplication", PLDI
// 1994, section 4).
struct FastDiv {
    unsigned m;
    int s;
};
inline FastDiv make_fastdiv(unsigned d)
{
    int l = 0;
    while ((1ull << l) < d) ++l;
    const unsigned long long p = 1ull << (31 + l);
    FastDiv f;
    f.m = (unsigned)((p + d - 1) / d);
    f.s = 31 + l;
    return f;
}
__host__ __device__ __forceinline__ unsigned fast_div(unsigned n, FastDiv d)
{
    return (unsigned)(((unsigned long long)n * d.m) >> d.s);
}

// A team of TPP = 32*WPP threads (16 for WPP = 0: two teams share a warp)
// owns one pencil; thread t holds the CPL
// cells c = m*TPP + t (m < CPL).  Cells >= n are padding: they compute on
// harmless values and are never reduced or stored.  NT > 0 is the pencil
// length known at compile time; when it equals the team's capacity (FULL)
// every slot is a cell and all index arithmetic folds into constants.
//
// Stencil exchange rows: one component of the pencil at cells -1 .. n+1,
// stored from row[-1], so the periodic neighbours c-1, c+1, c+2 of any cell
// are fixed offsets from c.  put() writes a cell and, for cells n-1, 0 and 1,
// their periodic copies at -1, n and n+1.  A row takes rs() = n+3 floats.
template <int CPL, int WPP, int NT = 0>
struct Team {
    static constexpr int TPP = team_threads<WPP>();
    static constexpr bool FULL = NT > 0 && NT == TPP * CPL;
    int t;      // thread within the team
    int n;      // pencil length

    __device__ void init(int t_, int n_)
    {
        t = t_;
        n = NT > 0 ? NT : n_;
    }
    __device__ __forceinline__ int len() const { return NT > 0 ? NT : n; }
    __device__ __forceinline__ int rs() const { return len() + 3; }
    __device__ __forceinline__ bool valid(int m) const { return FULL || m * TPP + t < len(); }
    // the slot's cell, or cell 0 for a padding slot (a safe address)
    __device__ __forceinline__ int ci(int m) const
    {
        return FULL ? m * TPP + t : (m * TPP + t < len() ? m * TPP + t : 0);
    }
    __device__ __forceinline__ void put(float *row, int m, float v) const
    {
        if (!valid(m)) return;
        const int c = m * TPP + t;
        const int nn = len();
        // a row holds cells -1 .. n+1 (the halo cells -1, n, n+1 included)
        if (MHD_SM(&row[c], 4) && MHD_IN(c, nn)) row[c] = v;
        if (FULL) {
            if (m == CPL - 1 && t == TPP - 1 && MHD_SM(&row[-1], 4)) row[-1] = v;
            if (m == 0 && t == 0 && MHD_SM(&row[nn], 4)) row[nn] = v;
            if (m == 0 && t == 1 && MHD_SM(&row[nn + 1], 4)) row[nn + 1] = v;
        } else {
            if (c == nn - 1 && MHD_SM(&row[-1], 4)) row[-1] = v;
            if (c == 0 && MHD_SM(&row[nn], 4)) row[nn] = v;
            if (c == (nn > 1 ? 1 : 0) && MHD_SM(&row[nn + 1], 4)) row[nn + 1] = v;
        }
    }

    // barrier over the team (and, when WPP > 1, over the CTA: every team of
    // a CTA runs the same phase sequence, so a CTA barrier is correct).
    __device__ __forceinline__ void sync() const
    {
        if (WPP <= 1) __syncwarp();   // a half-warp team's partner runs the same sequence
        else __syncthreads();
    }

    // max over the pencil of per-thread values (values >= 0; NaN ignored as
    // the reference's strict '>' scan from 0 ignores it).
    __device__ float pencil_max(float x, float *red) const
    {
#pragma unroll
        for (int o = (TPP < 32 ? TPP : 32) / 2; o > 0; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
        if (WPP <= 1) return x;
        const int w = t >> 5;
        if ((t & 31) == 0 && MHD_SM(&red[w], 4)) red[w] = x;
        __syncthreads();
        float r = MHD_SM(red, 4 * WPP) ? red[0] : 0.0f;
#pragma unroll
        for (int i = 1; i < WPP; ++i) r = fmaxf(r, MHD_SM(red, 4 * WPP) ? red[i] : 0.0f);
        __syncthreads();
        return r;
    }
};

// max over the CTA of non-negative values, then one atomicMax of the float's
// bit pattern (monotone for non-negative floats); NaN is dropped as the
// reference's strict '>' scan drops it.  Every thread of the CTA calls it.
__device__ __forceinline__ void cfl_block_max(float cl, unsigned *cmax)
{
    __shared__ float red[32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cl = fmaxf(cl, __shfl_xor_sync(0xffffffffu, cl, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = cl;
    __syncthreads();
    if (threadIdx.x == 0) {
        float r = red[0];
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) r = fmaxf(r, red[w]);
        atomicMax(cmax, __float_as_uint(r));
    }
    __syncthreads();
}

// The same fold from one warp, without a CTA barrier: a warp max, then one
// atomicMax by lane 0 unless the word already holds as much (a stale read only
// costs an extra atomic).  Every lane of the warp calls it.
__device__ __forceinline__ void cfl_warp_max(float cl, unsigned *cmax)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cl = fmaxf(cl, __shfl_xor_sync(0xffffffffu, cl, o));
    if ((threadIdx.x & 31) == 0 && cl > __uint_as_float(*(volatile unsigned *)cmax))
        atomicMax(cmax, __float_as_uint(cl));
}

// Device health word bits (also in include/mhdgpu.h).
__device__ __forceinline__ void flag_health(unsigned *health, unsigned bits)
{
    if (health) atomicOr(health, bits);
}

// Asynchronous 4-byte global -> shared copy (cp.async, no register round
// trip): a thread can have all of its staging copies in flight at once.
// Complete them with cp_async_wait_all() and then a barrier.  The issue
// carries no compiler memory clobber, so the staging loops keep their
// addresses in registers; the wait has one, and nothing touches a
// destination before its wait.
__device__ __forceinline__ void cp_async4(float *smem_dst, const float *gmem_src)
{
    if (!MHD_SM(smem_dst, 4)) return;
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem_src));
}

__device__ __forceinline__ void cp_async16(void *smem_dst, const void *gmem_src)
{
    if (!MHD_SM(smem_dst, 16)) return;
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem_dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem_src));
}

__device__ __forceinline__ void cp_async_wait_all()
{
    asm volatile("cp.async.wait_all;\n" ::: "memory");
}

// Cooperative copy of `count` floats, 16-byte vectors when both ends allow it.
// Coherent cp.async copies (the fluid kernels may run in place, so the
// source is not read-only for the kernel's lifetime); every copy of the
// calling thread is complete on return, the caller's barrier publishes them.
__device__ __forceinline__ void block_copy_in(float *__restrict__ dst, const float *__restrict__ src,
                                              long long count, int tid, int nthreads)
{
    const bool vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0
                     && (count & 3) == 0;
    if (vec) {
        const long long n4 = count >> 2;
        for (long long i = tid; i < n4; i += nthreads) cp_async16(dst + 4 * i, src + 4 * i);
    } else {
        for (long long i = tid; i < count; i += nthreads) cp_async4(dst + i, src + i);
    }
    cp_async_wait_all();
}

__device__ __forceinline__ void block_copy_out(float *__restrict__ dst, const float *__restrict__ src,
                                               long long count, int tid, int nthreads)
{
    const bool vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0
                     && (count & 3) == 0;
    if (vec) {
        const float4 *s4 = reinterpret_cast<const float4 *>(src);
        float4 *d4 = reinterpret_cast<float4 *>(dst);
        const long long n4 = count >> 2;
        for (long long i = tid; i < n4; i += nthreads)
            if (MHD_SM(s4 + i, 16)) d4[i] = s4[i];
    } else {
        for (long long i = tid; i < count; i += nthreads)
            if (MHD_SM(src + i, 4)) dst[i] = src[i];
    }
}

}  // namespace mhd
