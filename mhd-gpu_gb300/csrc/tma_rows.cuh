// tma_rows.cuh - TMA staging of the fluid tile's row-staged pencils (the y and
// z sweeps of the transpose-free step): one tensor copy per array brings the
// tile's rows into shared memory as they lie ([i][5P] floats of u, [i][3P+4]
// of b with the j+1 column, [i][3P] of b at plane k+1, [i][4] of b at column
// 0 when the j+1 column wraps), a shared-memory pass spreads them into the
// component-major layout the register-blocked tile computes on, and the
// updated u goes back the same way: gathered into [i][5P] rows and written by
// one tensor store.  The copies run in the TMA unit; the threads only spend
// the two shared-memory passes on them.
#pragma once

#include "kernels.cuh"
#include "tma.cuh"

#undef MHD_DBG_FILE
#define MHD_DBG_FILE 8

namespace mhd {

// pencils per tile of the TMA-staged fluid tile (the maps' box width)
constexpr int kTmaPencils = 8;

// the raw TMA area (floats) of a tile of n-cell pencils: u, b, b at k+1, b of
// column 0; every part a multiple of 32 floats (128 bytes) for n % 8 == 0
__host__ __device__ inline long long txr_raw_floats(int n)
{
    constexpr int P = kTmaPencils;
    return (long long)n * (5 * P + (3 * P + 4) + 3 * P + 4);
}
// the whole shared area: the cp.async layout of fluidx_reg.cuh, then the raw
// area at the next 128-byte boundary (32 floats of slack cover any alignment
// of the dynamic shared memory's start), then the mbarrier (8 bytes)
__host__ __device__ inline long long txr_smem_floats(long long fxr_floats, int n)
{
    return fxr_floats + 32 + txr_raw_floats(n) + 2;
}
// the raw area of a tile whose cp.async layout starts at smem
__device__ __forceinline__ float *txr_raw(float *smem, long long fxr_floats)
{
    const uintptr_t p = reinterpret_cast<uintptr_t>(smem + fxr_floats);
    return reinterpret_cast<float *>((p + 127) & ~static_cast<uintptr_t>(127));
}

// Stages the tile (pencils j0 .. j0+nvalid-1 of plane k, frame f) into US
// (component-major u), SB (b of columns j0 .. j0+nvalid, cell-major in frame
// order) and SK (frame b(3) of plane k+1) through TMA, then barriers.  Every
// thread of the CTA calls it.  Returns false when the copies did not complete
// within the bounded wait (the caller flags the box).
template <int N>
__device__ __forceinline__ bool tma_rows_stage(const Frame &f, const RowMaps &mp, float *US, int PS, int CS,
                                               float *SB, int BSR, float *SK, int KS, float *raw, uint64_t *bar,
                                               int j0, int k, int nvalid)
{
    constexpr int P = kTmaPencils;
    constexpr int WU = 5 * P, WB = 3 * P + 4, WK = 3 * P;
    float *RU = raw, *RB = RU + N * WU, *RK = RB + N * WB, *RW = RK + N * WK;
    const bool wrap = j0 + nvalid == f.ny;   // the last column's j+1 neighbour is column 0
    if (threadIdx.x == 0) {
        mbar_init(bar, 1);
        mbar_init_fence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        const unsigned bytes = 4u * N * (WU + WB + WK + (wrap ? 4 : 0));
        mbar_arrive_expect_tx(bar, bytes);
        const int kp = (k + 1 == f.nz) ? 0 : k + 1;
        tma_load_3d(RU, &mp.u, 5 * j0, 0, k, bar);
        tma_load_3d(RB, &mp.b, 3 * j0, 0, k, bar);
        tma_load_3d(RK, &mp.bk, 3 * j0, 0, kp, bar);
        if (wrap) tma_load_3d(RW, &mp.bw, 0, 0, k, bar);
    }
    bool ok = mbar_wait(bar, 0);
    if (!ok) ok = mbar_wait(bar, 0);   // give the copies a second bounded wait before reading
    // u: [i][5P] rows (stored components) -> US[q][frame component][i].  A
    // warp takes one 16-byte column w of 32 consecutive rows: lane l reads
    // row i0+l and writes its four floats to four component rows, so
    // consecutive lanes write consecutive banks.
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
        const float4 *R4 = reinterpret_cast<const float4 *>(RU);
        constexpr int NB = (N + 31) / 32;
        for (int pr = warp; pr < NB * (WU / 4); pr += nwarps) {
            const int w = pr % (WU / 4), i = (pr / (WU / 4)) * 32 + lane;
            if (i >= N) continue;
            if (!MHD_SM(&R4[i * (WU / 4) + w], 16)) continue;
            const float4 v = R4[i * (WU / 4) + w];
            const float e4[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int idx = 4 * w + e, qq = idx / 5, s = idx - 5 * qq;
                if (qq < nvalid && MHD_SM(&US[qq * PS + nib(f.iu, s) * CS + i], 4))
                    US[qq * PS + nib(f.iu, s) * CS + i] = e4[e];
            }
        }
    }
    // b of columns j0 .. j0+P (the column after the last valid one is its
    // periodic j+1 neighbour: column 0 when the tile ends the frame) ->
    // SB[qb][3 i + frame component]; columns past it are spare
    {
        constexpr int RBW = 3 * (P + 1);
        for (int h = threadIdx.x; h < N * RBW; h += blockDim.x) {
            const int i = h / RBW, r = h - i * RBW, qb = r / 3, s = r - 3 * qb;
            const float *src = (wrap && qb == nvalid) ? &RW[i * 4 + s] : &RB[i * WB + r];
            if (MHD_SM(src, 4) && MHD_SM(&SB[qb * BSR + 3 * i + nib(f.ib, s)], 4))
                SB[qb * BSR + 3 * i + nib(f.ib, s)] = *src;
        }
    }
    // frame b(3) of plane k+1 -> SK[q][i]
    {
        const int s3 = nib(f.pb, 2);
        for (int h = threadIdx.x; h < N * P; h += blockDim.x) {
            const int qq = h / N, i = h - qq * N;
            if (MHD_SM(&SK[qq * KS + i], 4) && MHD_SM(&RK[i * WK + 3 * qq + s3], 4))
                SK[qq * KS + i] = RK[i * WK + 3 * qq + s3];
        }
    }
    __syncthreads();
    return ok;
}

// Writes the tile's updated u (US, component-major) back through one tensor
// store: gathered into [i][5P] rows of stored components in the raw area,
// then stored by thread 0, which waits until the store has read the rows.
// Columns beyond the frame (a partial last tile) fall outside the tensor and
// are not written.  Every thread calls it after the update of US.
template <int N>
__device__ __forceinline__ void tma_rows_writeback(const Frame &f, const RowMaps &mp, const float *US, int PS,
                                                   int CS, float *raw, int j0, int k, int nvalid)
{
    constexpr int P = kTmaPencils;
    constexpr int WU = 5 * P;
    float4 *R4 = reinterpret_cast<float4 *>(raw);
    __syncthreads();
    {
        // the u transpose's mapping, the other way
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
        constexpr int NB = (N + 31) / 32;
        for (int pr = warp; pr < NB * (WU / 4); pr += nwarps) {
            const int w = pr % (WU / 4), i = (pr / (WU / 4)) * 32 + lane;
            if (i >= N) continue;
            float e4[4];
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int idx = 4 * w + e, qq = idx / 5, s = idx - 5 * qq;
                e4[e] = qq < nvalid && MHD_SM(&US[qq * PS + nib(f.iu, s) * CS + i], 4)
                            ? US[qq * PS + nib(f.iu, s) * CS + i] : 0.0f;
            }
            if (MHD_SM(&R4[i * (WU / 4) + w], 16)) R4[i * (WU / 4) + w] = make_float4(e4[0], e4[1], e4[2], e4[3]);
        }
    }
    fence_proxy_async_smem();
    __syncthreads();
    if (threadIdx.x == 0) {
        tma_store_3d(&mp.u, 5 * j0, 0, k, raw);
        bulk_commit();
        bulk_wait_read();
    }
}

}  // namespace mhd
