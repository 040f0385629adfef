// fluidx_reg.cuh - the fluid sweep, register-blocked, for pencils whose length
// fills a team of at most one warp exactly (n = 32*CPL, or 16*CPL for
// half-warp teams): the 32, 48, 64, 96 and 128-cell pencils.
//
// Algorithm and rounding: exactly fluidx_tile's (fluidx_kernel.cuh; reference
// Heterogeneous_MHD/C/fluidx.c:19-102, tvd1.c:8-118, mhdflux.c:9-72),
// operation for operation, so the two give the same bits.  Only the data
// movement differs:
//  - thread t of a team owns the consecutive cells t*CPL .. t*CPL+CPL-1, so a
//    stencil neighbour (i-1, i+1, i+2) is in the thread's own registers or, at
//    the ends of its run, in the adjacent lane's, fetched with a warp shuffle;
//    lane 0's left neighbour is lane TPP-1, which is the pencil's periodic
//    wrap;
//  - each difference of the limiter is formed once and used by both cells
//    that need it, and fl = c*wl once per cell;
//  - u is staged component-major per pencil ([pencil][component][cell], rows
//    of n+4 floats), so a thread reads or writes one component of its run with
//    one vector access; b stays cell-major;
//  - there are no exchange rows in shared memory and no team barriers.
#pragma once

#include <type_traits>

#include "kernels.cuh"
#include "tma_rows.cuh"

#undef MHD_DBG_FILE
#define MHD_DBG_FILE 1

namespace mhd {

// floats of u and of b of a frame's box (the extents the debug build checks
// global indices against)
#define MHD_NU(f) (5LL * (f).npen * (f).n)
#define MHD_NB(f) (3LL * (f).npen * (f).n)

// shared-memory geometry (floats); every offset is a multiple of 4 floats
__host__ __device__ inline int fxr_cs(int n) { return n + 4; }                    // a component of u
__host__ __device__ inline int fxr_ps(int n) { return 5 * fxr_cs(n); }            // u of one pencil
__host__ __device__ inline int fxr_bs(int n, bool rows) { return rows ? 3 * n + 4 : 3 * n; }   // b of one pencil
__host__ __device__ inline int fxr_ks(int n) { return n + 4; }                    // rows: b(3) of the k+1 pencil
__host__ __device__ inline long long fxr_smem_floats(int n, int ppc, bool rows)
{
    long long s = (long long)ppc * fxr_ps(n);
    if (rows) s += (long long)(ppc + 1) * fxr_bs(n, true) + (long long)ppc * fxr_ks(n);
    else s += (long long)ppc * fxr_bs(n, false);
    return s;
}

// the lanes of one team (TPP = 16 or 32 consecutive lanes of a warp)
template <int TPP>
struct Lanes {
    int t;   // lane within the team
    // v of lane t+d of the team, periodic.  Every lane of the warp calls it.
    __device__ __forceinline__ float from(float v, int d) const
    {
        return __shfl_sync(0xffffffffu, v, (t + d + TPP) & (TPP - 1), TPP);
    }
    // max over the team (values >= 0; NaN dropped as Team::pencil_max drops it)
    __device__ __forceinline__ float max(float x) const
    {
#pragma unroll
        for (int o = TPP / 2; o > 0; o >>= 1) x = fmaxf(x, __shfl_xor_sync(0xffffffffu, x, o));
        return x;
    }
};

// K consecutive floats at p in shared memory: 16-byte accesses for K % 4 == 0,
// 8-byte for K % 2 == 0 (p is aligned accordingly by the geometry above)
template <int K>
__device__ __forceinline__ void lds_run(const float *p, float (&v)[K])
{
    if (!MHD_SM(p, 4 * K)) {
#pragma unroll
        for (int i = 0; i < K; ++i) v[i] = 0.0f;
        return;
    }
    if constexpr (K % 4 == 0) {
#pragma unroll
        for (int i = 0; i < K / 4; ++i) {
            const float4 x = reinterpret_cast<const float4 *>(p)[i];
            v[4 * i] = x.x; v[4 * i + 1] = x.y; v[4 * i + 2] = x.z; v[4 * i + 3] = x.w;
        }
    } else if constexpr (K % 2 == 0) {
#pragma unroll
        for (int i = 0; i < K / 2; ++i) {
            const float2 x = reinterpret_cast<const float2 *>(p)[i];
            v[2 * i] = x.x; v[2 * i + 1] = x.y;
        }
    } else {
#pragma unroll
        for (int i = 0; i < K; ++i) v[i] = p[i];
    }
}

template <int K>
__device__ __forceinline__ void sts_run(float *p, const float (&v)[K])
{
    if (!MHD_SM(p, 4 * K)) return;
    if constexpr (K % 4 == 0) {
#pragma unroll
        for (int i = 0; i < K / 4; ++i)
            reinterpret_cast<float4 *>(p)[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
    } else if constexpr (K % 2 == 0) {
#pragma unroll
        for (int i = 0; i < K / 2; ++i) reinterpret_cast<float2 *>(p)[i] = make_float2(v[2 * i], v[2 * i + 1]);
    } else {
#pragma unroll
        for (int i = 0; i < K; ++i) p[i] = v[i];
    }
}

// component ii of the thread's run of u, or of the default state
// (1, 0, 0, 0, 1) for a pencil that is not live (it computes on harmless
// values and stores nothing)
template <int CPL>
__device__ __forceinline__ void load_comp(const float *p, bool live, int ii, float (&v)[CPL])
{
    if (live) {
        lds_run<CPL>(p, v);
    } else {
#pragma unroll
        for (int m = 0; m < CPL; ++m) v[m] = (ii == 0 || ii == 4) ? 1.0f : 0.0f;
    }
}

// Vector rows staging.  A tile's row i is ppc consecutive cells of the frame's
// j axis, contiguous in memory: 20 ppc bytes of u and 12 ppc of b.  When the
// tile is full (ppc pencils, ppc a multiple of 4) and every row starts on a
// 16-byte boundary (the frame's strides and the arrays' addresses multiples
// of 4 cells, resp. 16 bytes), a thread moves a quad of four pencils of one
// row with 16-byte accesses: five vectors of u, three of b, and scatters the
// 20 + 12 floats to their component-major places with offsets fixed by the
// quad's position (a handful of instructions per cell, against a warp pass
// per row of per-lane 4-byte copies otherwise).  Consecutive threads take
// consecutive rows, so the shared-memory stores are free of bank conflicts.
__device__ __forceinline__ bool rows_vec_ok(const Frame &f, int ppc, int nvalid, const float *u_in,
                                            const float *u_out, const float *b)
{
    const uintptr_t al = reinterpret_cast<uintptr_t>(u_in) | reinterpret_cast<uintptr_t>(u_out) |
                         reinterpret_cast<uintptr_t>(b);
    return nvalid == ppc && (ppc & 3) == 0 && ((f.si | f.sk) & 3) == 0 && (al & 15u) == 0;
}

// one quad of u (four pencils of row i, cells j0 + 4Q ..) -> US (its rows of
// the component-major layout at d = US + 4Q PS + i); co[s] = frame row of
// stored component s times CS
template <int PS>
__device__ __forceinline__ void rows_vec_put_u(float *d, const float4 (&v)[5], const int (&co)[5])
{
    const float e[20] = {v[0].x, v[0].y, v[0].z, v[0].w, v[1].x, v[1].y, v[1].z, v[1].w, v[2].x, v[2].y,
                         v[2].z, v[2].w, v[3].x, v[3].y, v[3].z, v[3].w, v[4].x, v[4].y, v[4].z, v[4].w};
#pragma unroll
    for (int x = 0; x < 20; ++x)
        if (MHD_SM(&d[(x / 5) * PS + co[x % 5]], 4)) d[(x / 5) * PS + co[x % 5]] = e[x];
}

template <int N>
__device__ __forceinline__ void rows_vec_stage(const Frame &f, const float *u_in, const float *b, float *US,
                                               float *SB, float *SK, int j0, int k, int ppc)
{
    constexpr int CS = N + 4, PS = 5 * CS, BSR = 3 * N + 4, KS = N + 4;
    const long long kb = (long long)k * f.sk;
    const int kp = (k + 1 == f.nz) ? 0 : k + 1;
    const long long kpb = (long long)kp * f.sk;
    const int pb2 = nib(f.pb, 2);
    int co[5], cb[3];
#pragma unroll
    for (int s = 0; s < 5; ++s) co[s] = nib(f.iu, s) * CS;
#pragma unroll
    for (int s = 0; s < 3; ++s) cb[s] = nib(f.ib, s);
    const int units = N * (ppc >> 2);
    for (int un = threadIdx.x; un < units; un += blockDim.x) {
        const int Q = un / N, i = un - Q * N;
        const long long cell = kb + (long long)i * f.si + j0 + 4 * Q;
        const float *gk = b + (kpb + (long long)i * f.si + j0 + 4 * Q) * 3 + pb2;
        if (!(MHD_GM(u_in + cell * 5, u_in, MHD_NU(f)) && MHD_GM(u_in + cell * 5 + 19, u_in, MHD_NU(f)) &&
              MHD_GM(b + cell * 3, b, MHD_NB(f)) && MHD_GM(b + cell * 3 + 11, b, MHD_NB(f)) &&
              MHD_GM(gk, b, MHD_NB(f)) && MHD_GM(gk + 9, b, MHD_NB(f))))
            continue;
        // every load of the quad first (all in flight together), then the stores
        float4 v[5];
        const float4 *gu = reinterpret_cast<const float4 *>(u_in + cell * 5);
#pragma unroll
        for (int w = 0; w < 5; ++w) v[w] = gu[w];
        const float4 *gb = reinterpret_cast<const float4 *>(b + cell * 3);
        const float4 w0 = gb[0], w1 = gb[1], w2 = gb[2];
        float kv[4];
#pragma unroll
        for (int x = 0; x < 4; ++x) kv[x] = gk[3 * x];
        rows_vec_put_u<PS>(US + 4 * Q * PS + i, v, co);
        {
            const float e[12] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w, w2.x, w2.y, w2.z, w2.w};
            float *d = SB + 4 * Q * BSR + 3 * i;
#pragma unroll
            for (int x = 0; x < 12; ++x)
                if (MHD_SM(&d[(x / 3) * BSR + cb[x % 3]], 4)) d[(x / 3) * BSR + cb[x % 3]] = e[x];
        }
        {
            float *d = SK + 4 * Q * KS + i;
#pragma unroll
            for (int x = 0; x < 4; ++x)
                if (MHD_SM(&d[x * KS], 4)) d[x * KS] = kv[x];
        }
    }
    // b of the column after the tile (column 0 when the tile ends the frame),
    // the j+1 neighbour of its last pencil
    int jx = j0 + ppc;
    if (jx >= f.ny) jx -= f.ny;
    for (int h = threadIdx.x; h < 3 * N; h += blockDim.x) {
        const int s = h / N, i = h - s * N;
        const float *g = b + (kb + (long long)i * f.si + jx) * 3 + s;
        if (MHD_SM(&SB[ppc * BSR + 3 * i + cb[s]], 4) && MHD_GM(g, b, MHD_NB(f))) SB[ppc * BSR + 3 * i + cb[s]] = *g;
    }
}

// the write-back of a full tile: a thread gathers a quad of one row from the
// component-major rows and stores its 20 floats as five 16-byte vectors
template <int N>
__device__ __forceinline__ void rows_vec_writeback(const Frame &f, float *u_out, const float *US, int j0, int k,
                                                   int ppc)
{
    constexpr int CS = N + 4, PS = 5 * CS;
    const long long kb = (long long)k * f.sk;
    int co[5];
#pragma unroll
    for (int s = 0; s < 5; ++s) co[s] = nib(f.iu, s) * CS;
    const int units = N * (ppc >> 2);
    for (int un = threadIdx.x; un < units; un += blockDim.x) {
        const int Q = un / N, i = un - Q * N;
        const float *d = US + 4 * Q * PS + i;
        float e[20];
#pragma unroll
        for (int x = 0; x < 20; ++x)
            e[x] = MHD_SM(&d[(x / 5) * PS + co[x % 5]], 4) ? d[(x / 5) * PS + co[x % 5]] : 0.0f;
        float *go = u_out + (kb + (long long)i * f.si + j0 + 4 * Q) * 5;
        if (!(MHD_GM(go, u_out, MHD_NU(f)) && MHD_GM(go + 19, u_out, MHD_NU(f)))) continue;
        float4 *g = reinterpret_cast<float4 *>(go);
#pragma unroll
        for (int w = 0; w < 5; ++w) g[w] = make_float4(e[4 * w], e[4 * w + 1], e[4 * w + 2], e[4 * w + 3]);
    }
}

// GROUPED: rows mode moves its rows in groups of four with per-lane offsets
// fixed for the tile (fewer copy instructions, more registers held); the
// single-box kernels take it, the register-capped batch kernels do not.
// TMA: rows mode stages the tile and writes it back through tensor copies
// (tma_rows.cuh; tm holds the frame's maps, ppc = kTmaPencils, in place).
template <int CPL, int TPP, bool ROWS, bool GROUPED, bool TMA, class MP>
__device__ __forceinline__ bool fluidx_tile_reg_pass(const FluidxArgs &a, long long tile, const RowMaps *tm, MP &mp)
{
    constexpr int N = TPP * CPL;
    constexpr int CS = N + 4, PS = 5 * CS, BSC = 3 * N, BSR = 3 * N + 4, KS = N + 4;
    extern __shared__ __align__(16) float smem_r[];
    float *smem = smem_r;
    const Frame &f = a.f;
    const int ppc = blockDim.x / TPP;
    const int q = threadIdx.x / TPP;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const Lanes<TPP> ln{(int)(threadIdx.x & (TPP - 1))};
    const int c0 = ln.t * CPL;

    long long p0 = 0;          // !ROWS: first linear pencil
    int j0 = 0, k = 0;         // ROWS: first j and the plane
    int nvalid;
    if (!ROWS) {
        p0 = tile * ppc;
        nvalid = (int)min((long long)ppc, f.npen - p0);
    } else {
        const int njb = (f.ny + ppc - 1) / ppc;
        k = (int)(tile / njb);
        j0 = (int)(tile - (long long)k * njb) * ppc;
        nvalid = min(ppc, f.ny - j0);
    }
    const bool live = q < nvalid;
    const bool vec = ROWS && !TMA && rows_vec_ok(f, ppc, nvalid, a.u_in, a.u_out, a.b);
    const int jq = ROWS ? j0 + q : (live ? (int)((p0 + q) % f.ny) : 0);
    const int kq = ROWS ? k : (live ? (int)((p0 + q) / f.ny) : 0);

    float *US = smem;                       // ppc * PS, component-major
    float *us = US + q * PS + c0;           // component ii of the run: us + ii*CS
    float *BS = smem + ppc * PS;            // b staging
    const float dt = *a.dt;

    // ---- stage u (kept) and b; cell-centred B of the run ----
    float bc[CPL][3];
    const float *bjp = nullptr, *bkp = nullptr;   // !ROWS: b of the j+1 and k+1 pencils
    {
        float bo[3 * CPL], bj[CPL], bk[CPL];   // own b; b(2) at j+1; b(3) at k+1
        if (!ROWS) {
            const float *gu = a.u_in + p0 * 5 * N;
            const int cells = nvalid * N;
            for (int c = threadIdx.x; c < cells; c += blockDim.x) {
                const int qq = c / N, cc = c - qq * N;
                float *d = US + qq * PS + cc;
                const float *s = gu + (long long)c * 5;
#pragma unroll
                for (int ii = 0; ii < 5; ++ii)
                    if (MHD_GM(s + ii, a.u_in, MHD_NU(f))) cp_async4(d + ii * CS, s + ii);
            }
            // b as it lies; completes this thread's u copies too
            if (MHD_GM(a.b + p0 * 3 * N, a.b, MHD_NB(f)) &&
                MHD_GM(a.b + (p0 + nvalid) * 3 * N - 1, a.b, MHD_NB(f)))
                block_copy_in(BS, a.b + p0 * 3 * N, (long long)nvalid * 3 * N, threadIdx.x, blockDim.x);
            __syncthreads();
            const int jp = (jq + 1 == f.ny) ? 0 : jq + 1;
            const int kp = (kq + 1 == f.nz) ? 0 : kq + 1;
            bjp = a.b + ((long long)kq * f.ny + jp) * 3 * N;
            bkp = a.b + ((long long)kp * f.ny + jq) * 3 * N;
            if (live) {
                lds_run<3 * CPL>(BS + q * BSC + c0 * 3, bo);
#pragma unroll
                for (int m = 0; m < CPL; ++m) {
                    bj[m] = MHD_GM(bjp + (c0 + m) * 3 + 1, a.b, MHD_NB(f)) ? bjp[(c0 + m) * 3 + 1] : 0.0f;
                    bk[m] = MHD_GM(bkp + (c0 + m) * 3 + 2, a.b, MHD_NB(f)) ? bkp[(c0 + m) * 3 + 2] : 0.0f;
                }
            }
        } else {
            const long long kb = (long long)k * f.sk;
            const int kp = (k + 1 == f.nz) ? 0 : k + 1;
            const long long kpb = (long long)kp * f.sk;
            float *SB = BS;                          // (ppc+1) * BSR: b of columns j0 .. j0+nvalid
            float *SK = BS + (ppc + 1) * BSR;        // ppc * KS: b(3) of plane k+1, [pencil][i]
            if constexpr (TMA) {
                float *raw = txr_raw(smem, fxr_smem_floats(N, ppc, true));
                uint64_t *bar = reinterpret_cast<uint64_t *>(raw + txr_raw_floats(N));
                if (!tma_rows_stage<N>(f, *tm, US, PS, CS, SB, BSR, SK, KS, raw, bar, j0, k, nvalid))
                    flag_health(a.health, MHD_HEALTH_STALL);
            } else if (vec) {
                rows_vec_stage<N>(f, a.u_in, a.b, US, SB, SK, j0, k, ppc);
            } else if constexpr (GROUPED) {
                const int ru = 5 * nvalid, rb = 3 * (nvalid + 1);
                const int pb2 = nib(f.pb, 2);
                // Groups of 4 rows (cells i0 .. i0+3 of the tile's pencils, N is a
                // multiple of 4).  A row holds ru floats of u at u_in + (row cell +
                // j0)*5, rb floats of b (columns j0 .. j0+nvalid, the last one
                // periodic) and nvalid b(3) values of plane k+1.  Each source takes
                // its own passes of the warp (u: 4 ru <= 160 floats in five, b:
                // 4 rb <= 108 in four, plane k+1: 4 nvalid <= 32 in one); lane e of
                // pass s moves element 32 s + e of its source, at offsets from the
                // group's first row that are fixed per lane.
                int uso[5], ugo[5], bso[4], bgo[4];
                bool uon[5], bon[4];
#pragma unroll
                for (int s = 0; s < 5; ++s) {
                    const int e = lane + 32 * s;
                    const int ro = e / ru, r = e - ro * ru;
                    const int qq = r / 5, p = r - qq * 5;
                    uon[s] = ro < 4;
                    uso[s] = uon[s] ? qq * PS + nib(f.iu, p) * CS + ro : 0;
                    ugo[s] = uon[s] ? (int)(ro * f.si + j0) * 5 + r : 0;
                }
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    const int e = lane + 32 * s;
                    const int ro = e / rb, r = e - ro * rb;
                    const int qb = r / 3, pp = r - qb * 3;
                    int j = j0 + qb;
                    if (j >= f.ny) j -= f.ny;
                    bon[s] = ro < 4;
                    bso[s] = bon[s] ? qb * BSR + nib(f.ib, pp) + 3 * ro : 0;
                    bgo[s] = bon[s] ? (int)(ro * f.si + j) * 3 + pp : 0;
                }
                const int kro = lane / nvalid, kqq = lane - kro * nvalid;
                const bool kon = kro < 4;
                const int kso = kon ? kqq * KS + kro : 0;
                const int kgo = kon ? (int)(kro * f.si + j0 + kqq) * 3 + pb2 : 0;
                for (int i0 = 4 * warp; i0 < N; i0 += 4 * nwarps) {
                    const long long rowc = kb + (long long)i0 * f.si;    // cell of (i0, 0, k)
                    const float *gu = a.u_in + rowc * 5;
                    const float *gb = a.b + rowc * 3;
                    const float *gk = a.b + (kpb + (long long)i0 * f.si) * 3;
#pragma unroll
                    for (int s = 0; s < 5; ++s)
                        if (uon[s] && MHD_GM(gu + ugo[s], a.u_in, MHD_NU(f))) cp_async4(&US[uso[s] + i0], gu + ugo[s]);
#pragma unroll
                    for (int s = 0; s < 4; ++s)
                        if (bon[s] && MHD_GM(gb + bgo[s], a.b, MHD_NB(f))) cp_async4(&SB[bso[s] + 3 * i0], gb + bgo[s]);
                    if (kon && MHD_GM(gk + kgo, a.b, MHD_NB(f))) cp_async4(&SK[kso + i0], gk + kgo);
                }
            } else {
                const int ru = 5 * nvalid, rb = 3 * (nvalid + 1);
                const int pb2 = nib(f.pb, 2);
                // per-lane offsets, independent of the row: a row of u is ru floats
                // at u_in + (rowc + j0)*5, element r -> pencil r/5, stored component r%5
                int us_off[2], sb_off[2], gb_off[2];
                bool us_on[2], sb_on[2];
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int r = lane + 32 * h;
                    us_on[h] = r < ru;
                    const int qq = r / 5, p = r - qq * 5;
                    us_off[h] = qq * PS + nib(f.iu, p) * CS;
                    sb_on[h] = r < rb;
                    const int qb = r / 3, pp = r - qb * 3;
                    int j = j0 + qb;
                    if (j >= f.ny) j -= f.ny;
                    sb_off[h] = qb * BSR + nib(f.ib, pp);
                    gb_off[h] = j * 3 + pp;
                }
                const bool sk_on = lane < nvalid;
                for (int i = warp; i < N; i += nwarps) {
                    const long long rowc = kb + (long long)i * f.si;    // cell of (i, 0, k)
                    const float *gu = a.u_in + (rowc + j0) * 5;
                    const float *gb = a.b + rowc * 3;
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        if (us_on[h] && MHD_GM(gu + lane + 32 * h, a.u_in, MHD_NU(f)))
                            cp_async4(&US[us_off[h] + i], gu + lane + 32 * h);
                        if (sb_on[h] && MHD_GM(gb + gb_off[h], a.b, MHD_NB(f)))
                            cp_async4(&SB[sb_off[h] + i * 3], gb + gb_off[h]);
                    }
                    const float *gk = a.b + (kpb + (long long)i * f.si + j0 + lane) * 3 + pb2;
                    if (sk_on && MHD_GM(gk, a.b, MHD_NB(f))) cp_async4(&SK[lane * KS + i], gk);
                }
            }
            cp_async_wait_all();
            __syncthreads();
            if (live) {
                float bn[3 * CPL];
                lds_run<3 * CPL>(SB + q * BSR + c0 * 3, bo);
                lds_run<3 * CPL>(SB + (q + 1) * BSR + c0 * 3, bn);
#pragma unroll
                for (int m = 0; m < CPL; ++m) bj[m] = bn[m * 3 + 1];
                lds_run<CPL>(SK + q * KS + c0, bk);
            }
        }
        if (!live) {
#pragma unroll
            for (int m = 0; m < CPL; ++m) {
                bo[3 * m] = 0.0f; bo[3 * m + 1] = 0.0f; bo[3 * m + 2] = 0.0f;
                bj[m] = 0.0f; bk[m] = 0.0f;
            }
        }
        // b3x = b/2 ; b3x(1) += cshift(b3x(1),1) ; b3x(2) += b(2,jp)/2 ;
        // b3x(3) += b(3,kp)/2   (fluidx.c:71-81; the halvings are exact)
        const float nb0 = ln.from(bo[0], 1);   // b(1) of the cell after the run
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            const float bnext = (m + 1 < CPL) ? bo[3 * (m + 1)] : nb0;
            bc[m][0] = fadd(0.5f * bo[3 * m], 0.5f * bnext);
            bc[m][1] = fadd(0.5f * bo[3 * m + 1], 0.5f * bj[m]);
            bc[m][2] = fadd(0.5f * bo[3 * m + 2], 0.5f * bk[m]);
        }
    }

    const float hdt = 0.5f * dt;
    unsigned bad = 0;
    float cfl_c = 0.0f;   // the last x sweep: the CFL speed of the updated cells
    float u1[CPL][5];

    // ================= half step =================
    {
        float v[CPL][5];
        float cl = 0.0f;
        {
            float uc[5][CPL];
#pragma unroll
            for (int ii = 0; ii < 5; ++ii) load_comp<CPL>(us + ii * CS, live, ii, uc[ii]);
#pragma unroll
            for (int m = 0; m < CPL; ++m) {
                const float uu[5] = {uc[0][m], uc[1][m], uc[2][m], uc[3][m], uc[4][m]};
                float cs, p;
                cell_flux(mp, uu, bc[m], v[m], cs, p);
                cl = fmaxf(cl, cs);
            }
        }
        const float c = ln.max(cl);
        // v/c where c > 0 (mhdflux.c:48-57); where c = 0 the quotient by 1
        // leaves every finite v as it is, without a select per value
        const float cd = c > 0.0f ? c : 1.0f;
        const float yc = mp.recip(cd);
#pragma unroll
        for (int ii = 0; ii < 5; ++ii) {
            float uu[CPL], wl[CPL], fl[CPL];
            load_comp<CPL>(us + ii * CS, live, ii, uu);
            // fr = c(u + v/c) (kept in u1), wl = u - v/c
#pragma unroll
            for (int m = 0; m < CPL; ++m) {
                const float vv = mp.divy(v[m][ii], cd, yc);
                u1[m][ii] = mp.mul(c, mp.add(uu[m], vv));
                wl[m] = mp.sub(uu[m], vv);
            }
            // flux = (fr - c*cshift(wl,+1))/2
            const float wr = ln.from(wl[0], 1);
#pragma unroll
            for (int m = 0; m < CPL; ++m)
                fl[m] = 0.5f * mp.sub(u1[m][ii], mp.mul(c, (m + 1 < CPL) ? wl[m + 1] : wr));
            // u1 = u - (flux - cshift(flux,-1)) dt/2
            const float fm = ln.from(fl[CPL - 1], -1);
#pragma unroll
            for (int m = 0; m < CPL; ++m)
                u1[m][ii] = mp.add(uu[m], mp.mul(-hdt, mp.sub(fl[m], m > 0 ? fl[m - 1] : fm)));
        }
    }

    // ================= full step =================
    {
        float v[CPL][5];
        float cl = 0.0f;
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            float cs, p;
            cell_flux(mp, u1[m], bc[m], v[m], cs, p);
            cl = fmaxf(cl, cs);
            if (!(p > 0.0f)) bad |= MHD_HEALTH_PRESSURE;
        }
        const float c = ln.max(cl);
        // v/c where c > 0 (mhdflux.c:48-57); where c = 0 the quotient by 1
        // leaves every finite v as it is, without a select per value
        const float cd = c > 0.0f ? c : 1.0f;
        const float yc = mp.recip(cd);
        const float mdt = -dt;
        float ssum[CPL];
#pragma unroll
        for (int m = 0; m < CPL; ++m) ssum[m] = 0.0f;
#pragma unroll
        for (int ii = 0; ii < 5; ++ii) {
            // fr = c(u1 + v/c), fl = c wl = c(u1 - v/c) of the run
            float fr[CPL], fl[CPL];
#pragma unroll
            for (int m = 0; m < CPL; ++m) {
                const float vv = mp.divy(v[m][ii], cd, yc);
                fr[m] = mp.mul(c, mp.add(u1[m][ii], vv));
                fl[m] = mp.mul(c, mp.sub(u1[m][ii], vv));
            }
            // neighbours: fr of cells c0-1 and c0+CPL, fl of c0+CPL and c0+CPL+1
            const float frl = ln.from(fr[CPL - 1], -1);
            const float frr = ln.from(fr[0], 1);
            const float flr1 = ln.from(fl[0], 1);
            const float flr2 = (CPL >= 2) ? ln.from(fl[CPL >= 2 ? 1 : 0], 1) : ln.from(fl[0], 2);
            // dr[i] = fr(c0+i) - fr(c0+i-1), dl[i] = fl(c0+i) - fl(c0+i+1), i = 0 .. CPL
            float dr[CPL + 1], dl[CPL + 1];
#pragma unroll
            for (int i = 0; i <= CPL; ++i) {
                const float ra = (i < CPL) ? fr[i] : frr;
                const float rb = (i > 0) ? fr[i - 1] : frl;
                dr[i] = mp.sub(ra, rb);
                const float la = (i < CPL) ? fl[i] : flr1;
                const float lb = (i + 1 < CPL) ? fl[i + 1] : (i + 1 == CPL ? flr1 : flr2);
                dl[i] = mp.sub(la, lb);
            }
            // flux = (fr - fl + dfr - dfl)/2 with van Leer slopes (tvd1.c:54-112):
            // dfr = slope(fr(c+1)-fr(c), fr(c)-fr(c-1)),
            // dfl = slope(fl(c+1)-fl(c+2), fl(c)-fl(c+1)), fl0 = fl(c+1)
            float fx[CPL];
#pragma unroll
            for (int m = 0; m < CPL; ++m) {
                const float dfr = mp.slope(dr[m + 1], dr[m]);
                const float dfl = mp.slope(dl[m + 1], dl[m]);
                const float fl0 = (m + 1 < CPL) ? fl[m + 1] : flr1;
                fx[m] = 0.5f * mp.add(mp.sub(fr[m], fl0), mp.sub(dfr, dfl));
            }
            // u = u - (flux - cshift(flux,-1)) dt, written back into US
            const float fxl = ln.from(fx[CPL - 1], -1);
            float uu[CPL], un[CPL];
            load_comp<CPL>(us + ii * CS, live, ii, uu);
#pragma unroll
            for (int m = 0; m < CPL; ++m) {
                un[m] = mp.add(uu[m], mp.mul(mdt, mp.sub(fx[m], m > 0 ? fx[m - 1] : fxl)));
                ssum[m] += un[m];
                if (ii == 0 && !(un[m] > 0.0f)) bad |= MHD_HEALTH_DENSITY;
            }
            if (live) sts_run<CPL>(us + ii * CS, un);
        }
#pragma unroll
        for (int m = 0; m < CPL; ++m)
            if (!isfinite(ssum[m])) bad |= MHD_HEALTH_NONFINITE;
        // the last x sweep of a step: the CFL fast speed of the updated cells,
        // as cfl_cell_speed forms it
        if (!ROWS && a.cfl != nullptr) {
            const float *bs = BS + q * BSC + c0 * 3;   // this run's staged b
            const float nb0 = ln.from(live && MHD_SM(bs, 4) ? bs[0] : 0.0f, 1);
            if (live) {
#pragma unroll
                for (int m = 0; m < CPL; ++m) {
                    float um[5], bb[3];
#pragma unroll
                    for (int ii = 0; ii < 5; ++ii) um[ii] = MHD_SM(&us[ii * CS + m], 4) ? us[ii * CS + m] : 1.0f;
                    if (!MHD_SM(bs + 3 * m, 12) || !MHD_SM(bs + 3 * (m + 1 < CPL ? m + 1 : m), 4)) continue;
                    if (a.cfl_mode == MHD_CFL_C) {
                        bb[0] = bs[3 * m]; bb[1] = bs[3 * m + 1]; bb[2] = bs[3 * m + 2];
                        if constexpr (MP::kFlagged) cfl_c = fmaxf(cfl_c, cfl_speed_c_ff(um, bb, mp.nb));
                        else cfl_c = fmaxf(cfl_c, cfl_speed_c(um, bb));
                    } else {
                        const float bnext = (m + 1 < CPL) ? bs[3 * (m + 1)] : nb0;
                        bb[0] = fdiv(fadd(bs[3 * m], bnext), 2.0f);
                        if (!MHD_GM(bjp + (c0 + m) * 3 + 1, a.b, MHD_NB(f)) ||
                            !MHD_GM(bkp + (c0 + m) * 3 + 2, a.b, MHD_NB(f)))
                            continue;
                        bb[1] = fdiv(fadd(bs[3 * m + 1], bjp[(c0 + m) * 3 + 1]), 2.0f);
                        bb[2] = fdiv(fadd(bs[3 * m + 2], bkp[(c0 + m) * 3 + 2]), 2.0f);
                        cfl_c = fmaxf(cfl_c, cfl_speed_averaged(um, bb));
                    }
                }
            }
        }
    }

    // A flagged pass commits nothing when a lane of the CTA formed a value
    // near a rounding boundary: its caller computes the tile again exactly
    // (the inputs are still untouched in memory).
    if constexpr (MP::kFlagged) {
        if (__syncthreads_or(mp.nb ? 1 : 0)) return false;
    }
    if (!ROWS && a.cfl != nullptr) cfl_warp_max(cfl_c, a.cfl);   // every lane of the warp
    if (!live) bad = 0;
    if (bad) flag_health(a.health, bad);
    __syncthreads();
    // ---- write back: component-major shared rows -> the cell-major state ----
    if (!ROWS) {
        float *g = a.u_out + p0 * 5 * N;
        if ((reinterpret_cast<uintptr_t>(g) & 15u) == 0) {
            // a group of 4 consecutive cells of one pencil: its five component
            // runs are five 16-byte shared loads, its 20 floats five 16-byte
            // stores (the transpose happens in registers)
            const int ngroups = nvalid * (N / 4);
            for (int gi = threadIdx.x; gi < ngroups; gi += blockDim.x) {
                const int qq = gi / (N / 4), cc = 4 * (gi - qq * (N / 4));
                const float *src = US + qq * PS + cc;
                float4 c[5];
#pragma unroll
                for (int ii = 0; ii < 5; ++ii)
                    c[ii] = MHD_SM(src + ii * CS, 16) ? *reinterpret_cast<const float4 *>(src + ii * CS)
                                                      : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                float *go = g + (size_t)(qq * N + cc) * 5;
                if (!(MHD_GM(go, a.u_out, MHD_NU(f)) && MHD_GM(go + 19, a.u_out, MHD_NU(f)))) continue;
                float4 *dst = reinterpret_cast<float4 *>(go);
                dst[0] = make_float4(c[0].x, c[1].x, c[2].x, c[3].x);
                dst[1] = make_float4(c[4].x, c[0].y, c[1].y, c[2].y);
                dst[2] = make_float4(c[3].y, c[4].y, c[0].z, c[1].z);
                dst[3] = make_float4(c[2].z, c[3].z, c[4].z, c[0].w);
                dst[4] = make_float4(c[1].w, c[2].w, c[3].w, c[4].w);
            }
        } else {
            const int nf = nvalid * 5 * N;
            for (int e = threadIdx.x; e < nf; e += blockDim.x) {
                const int cell = e / 5, comp = e - 5 * cell, qq = cell / N, cc = cell - qq * N;
                if (MHD_SM(&US[qq * PS + comp * CS + cc], 4) && MHD_GM(g + e, a.u_out, MHD_NU(f)))
                    g[e] = US[qq * PS + comp * CS + cc];
            }
        }
    } else {
        if constexpr (TMA) {
            float *raw = txr_raw(smem, fxr_smem_floats(N, ppc, true));
            tma_rows_writeback<N>(f, *tm, US, PS, CS, raw, j0, k, nvalid);
        } else if (vec) {
            rows_vec_writeback<N>(f, a.u_out, US, j0, k, ppc);
        } else if constexpr (GROUPED) {
            // groups of 4 rows: a row is ru = 5*nvalid consecutive floats at
            // u_out + (row cell + j0)*5; the 4*ru <= 160 floats of a group take
            // five passes of a warp, each lane with fixed (row, pencil, component)
            const long long kb = (long long)k * f.sk;
            const int ru = 5 * nvalid;
            int so[5], go[5];
            bool on[5];
#pragma unroll
            for (int s = 0; s < 5; ++s) {
                const int e = lane + 32 * s;
                const int ro = e / ru, r = e - ro * ru;
                const int qq = r / 5, p = r - qq * 5;
                on[s] = ro < 4;
                so[s] = on[s] ? qq * PS + nib(f.iu, p) * CS + ro : 0;
                go[s] = on[s] ? (int)(ro * f.si + j0) * 5 + r : 0;
            }
            for (int i0 = 4 * warp; i0 < N; i0 += 4 * nwarps) {
                float *g = a.u_out + (kb + (long long)i0 * f.si) * 5;
#pragma unroll
                for (int s = 0; s < 5; ++s)
                    if (on[s] && MHD_SM(&US[so[s] + i0], 4) && MHD_GM(g + go[s], a.u_out, MHD_NU(f)))
                        g[go[s]] = US[so[s] + i0];
            }
        } else {
            const long long kb = (long long)k * f.sk;
            const int ru = 5 * nvalid;
            int off[2];
            bool on[2];
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                const int r = lane + 32 * h;
                on[h] = r < ru;
                const int qq = r / 5, p = r - qq * 5;
                off[h] = qq * PS + nib(f.iu, p) * CS;
            }
            for (int i = warp; i < N; i += nwarps) {
                float *g = a.u_out + (kb + (long long)i * f.si + j0) * 5;
#pragma unroll
                for (int h = 0; h < 2; ++h)
                    if (on[h] && MHD_SM(&US[off[h] + i], 4) && MHD_GM(g + lane + 32 * h, a.u_out, MHD_NU(f)))
                        g[lane + 32 * h] = US[off[h] + i];
            }
        }
    }
    return true;
}

// the exact pass of a flagged tile, after the flagged pass: its FP64
// fallbacks' calls sit outside the flagged pass's hot code (inlined: out of
// line, as a call of its own, it measured 0.5 % slower on the batched step)
template <int CPL, int TPP, bool ROWS, bool GROUPED, bool TMA>
__device__ __forceinline__ void fluidx_tile_reg_exact(const FluidxArgs &a, long long tile, const RowMaps *tm)
{
    Faithful m;
    fluidx_tile_reg_pass<CPL, TPP, ROWS, GROUPED, TMA>(a, tile, tm, m);
}

// One tile of the fluid sweep.  FLAGGED (the batched kernels): Faithful (the
// C path's rounding) runs first as FaithfulNB, without its FP64 fallbacks in
// the hot code, and the rare tile in which a value lies near a rounding
// boundary is computed again with them.  The single-box kernels call the
// fallbacks in place: on smooth single-box states (a linear wave) the
// near-boundary values come in whole regions and the redos cost more than
// the calls.
template <int CPL, int TPP, class M, bool ROWS, bool GROUPED = false, bool TMA = false, bool FLAGGED = false>
__device__ __forceinline__ void fluidx_tile_reg(const FluidxArgs &a, long long tile, const RowMaps *tm = nullptr)
{
    if constexpr (FLAGGED && std::is_same<M, Faithful>::value) {
        FaithfulNB f;
        if (!fluidx_tile_reg_pass<CPL, TPP, ROWS, GROUPED, TMA>(a, tile, tm, f)) {
            __syncthreads();   // the flagged pass's shared memory is consumed
            fluidx_tile_reg_exact<CPL, TPP, ROWS, GROUPED, TMA>(a, tile, tm);
        }
    } else {
        M m;
        fluidx_tile_reg_pass<CPL, TPP, ROWS, GROUPED, TMA>(a, tile, tm, m);
    }
}

}  // namespace mhd
