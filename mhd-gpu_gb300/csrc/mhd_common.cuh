// mhd_common.cuh - shared device plumbing for the sm_103a MHD kernels:
// pencil geometry, the pencil-team (one or more warps that own one pencil),
// neighbour exchange through shared memory, pencil-wide max reduction and the
// device health word.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "mhd_math.cuh"
#include "../../include/mhdgpu.h"

namespace mhd {

// Pencil geometry of one frame in the reference layout u(5,n,ny,nz),
// b(3,n,ny,nz): the pencil runs along the fastest spatial axis (length n),
// pencil index p = j + ny*k.
struct Frame {
    int n, ny, nz;
    long long npen;
};

__host__ __device__ inline Frame make_frame(int n, int ny, int nz)
{
    Frame f;
    f.n = n; f.ny = ny; f.nz = nz;
    f.npen = (long long)ny * (long long)nz;
    return f;
}

// A team of TPP = 32*WPP threads owns one pencil; thread t holds the CPL
// cells c = m*TPP + t (m < CPL).  Cells >= n are padding: they compute on
// harmless values and are never reduced or stored.
template <int CPL, int WPP>
struct Team {
    static constexpr int TPP = 32 * WPP;
    int t;      // thread within the team
    int n;      // pencil length
    int cell[CPL];
    int ip[CPL], im[CPL], ipp[CPL];
    bool valid[CPL];

    __device__ void init(int t_, int n_)
    {
        t = t_;
        n = n_;
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            int c = m * TPP + t;
            valid[m] = c < n;
            if (!valid[m]) c = 0;
            cell[m] = c;
            int a = c + 1; if (a >= n) a -= n;
            int b = a + 1; if (b >= n) b -= n;
            ip[m] = a;
            ipp[m] = b;
            im[m] = (c == 0) ? n - 1 : c - 1;
        }
    }

    // barrier over the team (and, when WPP > 1, over the CTA: every team of
    // a CTA runs the same phase sequence, so a CTA barrier is correct).
    __device__ __forceinline__ void sync() const
    {
        if (WPP == 1) __syncwarp();
        else __syncthreads();
    }

    // max over the pencil of per-thread values (values >= 0; NaN ignored as
    // the reference's strict '>' scan from 0 ignores it).
    __device__ float pencil_max(float x, float *red) const
    {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
        if (WPP == 1) return x;
        const int w = t >> 5;
        if ((t & 31) == 0) red[w] = x;
        __syncthreads();
        float r = red[0];
#pragma unroll
        for (int i = 1; i < WPP; ++i) r = fmaxf(r, red[i]);
        __syncthreads();
        return r;
    }
};

// Device health word bits (also in include/mhdgpu.h).
__device__ __forceinline__ void flag_health(unsigned *health, unsigned bits)
{
    if (health) atomicOr(health, bits);
}

// Cooperative copy of `count` floats, 16-byte vectors when both ends allow it.
// Plain (coherent) loads: the fluid kernels may run in place, so the source
// is not read-only for the kernel's lifetime.
__device__ __forceinline__ void block_copy_in(float *__restrict__ dst, const float *__restrict__ src,
                                              long long count, int tid, int nthreads)
{
    const bool vec = ((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0
                     && (count & 3) == 0;
    if (vec) {
        const float4 *s4 = reinterpret_cast<const float4 *>(src);
        float4 *d4 = reinterpret_cast<float4 *>(dst);
        const long long n4 = count >> 2;
        for (long long i = tid; i < n4; i += nthreads) d4[i] = s4[i];
    } else {
        for (long long i = tid; i < count; i += nthreads) dst[i] = src[i];
    }
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
        for (long long i = tid; i < n4; i += nthreads) d4[i] = s4[i];
    } else {
        for (long long i = tid; i < count; i += nthreads) dst[i] = src[i];
    }
}

}  // namespace mhd
