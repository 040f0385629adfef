// fluidx_kernel.cuh - the fluid sweep (relaxing TVD, RK2) on pencils of a
// frame view, for sm_103a.  Instantiated per math policy and staging mode in
// fluidx.cu (faithful) and fluidx_fast.cu (fast).
//
// Algorithm: Heterogeneous_MHD/C/fluidx.c:19-102 (gather + cell-centred B),
// tvd1.c:8-118 (RK2 half and full step, van Leer limiter), mhdflux.c:9-72
// (flux vector and pencil-wide max fast speed).
//
// GB300 mapping.  A CTA owns PPC pencils and stages their u into shared
// memory (US), where it stays for the whole update and receives the result;
// registers hold only the cell-centred B, the half-step state and the fluxes
// of the cells a thread owns.  Two staging modes:
//   ROWS = false: the pencils are contiguous (si = 1: the reference layout, or
//     the x sweep of an x-major box); the CTA's pencils are consecutive, so u
//     and b are single contiguous chunks moved with 16-byte accesses;
//   ROWS = true: the pencils run across memory (sj = 1: the y and z sweeps of
//     an x-major box, read in place instead of after a transpose); the CTA owns
//     PPC neighbouring pencils at one k, so each cell i of them is one
//     contiguous row of PPC cells, and rows are moved with consecutive lanes
//     on consecutive addresses (the transpose happens in shared memory).
// Two tiles with the same arithmetic: for pencils that fill a team of at most
// one warp exactly (32, 48, 64, 96, 128 cells) the register-blocked tile of
// fluidx_reg.cuh (thread t owns consecutive cells, neighbours by warp
// shuffle); for every other length the team tile below, where each pencil
// belongs to a team of 32*WPP threads, CPL cells per thread (cell
// c = m*32*WPP + t), stencil neighbours (i-1, i+1, i+2) go through a
// per-pencil shared buffer and the two pencil-wide maxima of the fast speed
// are warp-shuffle reductions (plus one shared step when WPP > 1).  No tensor
// cores: nothing on this path is a contraction; the kernel is bounded by
// instruction issue.
#pragma once

#include "fluidx_reg.cuh"
#include "kernels.cuh"

#undef MHD_DBG_FILE
#define MHD_DBG_FILE 2

namespace mhd {

// shared-memory geometry (floats), shared by the kernel and its launcher
__host__ __device__ inline int fx_ps(int n, bool rows)          // u stride per pencil
{
    return rows ? 5 * n + ((37 - (5 * n) % 32) % 32) : 5 * n;   // = 5 (mod 32) for rows
}
__host__ __device__ inline int fx_bs(int n) { return 3 * n + ((35 - (3 * n) % 32) % 32); }
// exchange area of one pencil: 10 halo rows of n+3 floats
__host__ __device__ inline long long fx_xpen(int n) { return 10LL * (n + 3); }
__host__ __device__ inline long long fx_xsize(int n, int ppc, bool rows)
{
    long long x = fx_xpen(n) * ppc;
    if (rows) {
        const long long need = (long long)(ppc + 1) * fx_bs(n) + (long long)(ppc + 1) * n;
        if (need > x) x = need;
    }
    return x;
}
__host__ __device__ inline long long fx_smem_floats(int n, int ppc, int wpp, bool rows)
{
    return (long long)ppc * fx_ps(n, rows) + fx_xsize(n, ppc, rows) + (long long)ppc * wpp;
}
// shared floats of the tile that a (cpl, wpp) team takes for pencils of n
// cells: register-blocked (fluidx_reg.cuh) when the pencil fills the team
__host__ __device__ inline long long fx_tile_smem_floats(int n, int ppc, int cpl, int wpp, bool rows)
{
    return reg_tile_shape(n, cpl, wpp) ? fxr_smem_floats(n, ppc, rows) : fx_smem_floats(n, ppc, wpp, rows);
}

// One CTA's work: tile = the CTA's group of pencils (contiguous mode: pencils
// tile*ppc ..; rows mode: j-block tile % njb of plane tile / njb), for any
// pencil length up to the team's capacity.  fluidx_tile below picks it or the
// register-blocked tile.
template <int CPL, int WPP, class M, bool ROWS, int NT>
__device__ __forceinline__ void fluidx_tile_team(const FluidxArgs &a, long long tile)
{
    constexpr int TPP = team_threads<WPP>();
    extern __shared__ float smem[];
    const Frame &f = a.f;
    const int n = NT > 0 ? NT : f.n;
    const int ppc = blockDim.x / TPP;
    const int q = threadIdx.x / TPP;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int ps = fx_ps(n, ROWS);

    // pencils of this CTA
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
    const int jq = ROWS ? j0 + q : (live ? (int)((p0 + q) % f.ny) : 0);
    const int kq = ROWS ? k : (live ? (int)((p0 + q) / f.ny) : 0);

    float *US = smem;                                       // ppc * ps
    float *XA = smem + (size_t)ppc * ps;                    // fx_xsize
    float *red = XA + fx_xsize(n, ppc, ROWS);               // ppc * WPP
    float *us = US + (size_t)q * ps;
    float *rq = red + q * WPP;

    Team<CPL, WPP, NT> tm;
    tm.init(threadIdx.x - q * TPP, n);
    const float dt = *a.dt;
    // exchange rows of this pencil: X(r)[c] for c in -1 .. n+1
    const int rs = tm.rs();
    float *x = XA + (size_t)q * fx_xpen(n) + 1;
    auto X = [&](int r) { return x + r * rs; };
    // value of exchange row r at cell i (-1 <= i <= n+1), of the staged u
    auto XR = [&](int r, int i) { return (MHD_IN(i + 1, rs) && MHD_SM(X(r) + i, 4)) ? X(r)[i] : 0.0f; };
    auto UR = [&](int i) { return MHD_SM(us + i, 4) ? us[i] : 0.0f; };
    (void)UR;

    // ---- stage u (kept) and b (transient) ----
    float bc[CPL][3];
    const float *bjp = nullptr, *bkp = nullptr;   // !ROWS: b of the j+1 and k+1 pencils
    if (!ROWS) {
        if (MHD_GM(a.u_in + p0 * 5 * n, a.u_in, MHD_NU(f)) &&
            MHD_GM(a.u_in + (p0 + nvalid) * 5 * n - 1, a.u_in, MHD_NU(f)))
            block_copy_in(US, a.u_in + p0 * 5 * n, (long long)nvalid * 5 * n, threadIdx.x, blockDim.x);
        if (MHD_GM(a.b + p0 * 3 * n, a.b, MHD_NB(f)) && MHD_GM(a.b + (p0 + nvalid) * 3 * n - 1, a.b, MHD_NB(f)))
            block_copy_in(XA, a.b + p0 * 3 * n, (long long)nvalid * 3 * n, threadIdx.x, blockDim.x);
        __syncthreads();
        // b3x = b/2 ; b3x(1) += cshift(b3x(1),1) ; b3x(2) += b(2,jp)/2 ;
        // b3x(3) += b(3,kp)/2   (fluidx.c:71-81; the halvings are exact).
        // Plain coherent loads, not the read-only path: the batched sweep
        // kernel writes b earlier in the same launch.
        const int jp = (jq + 1 == f.ny) ? 0 : jq + 1;
        const int kp = (kq + 1 == f.nz) ? 0 : kq + 1;
        bjp = a.b + ((long long)kq * f.ny + jp) * 3 * n;
        bkp = a.b + ((long long)kp * f.ny + jq) * 3 * n;
        const float *pb = XA + (size_t)q * 3 * n;
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            const int c = tm.ci(m);
            const int cp = (c + 1 == n) ? 0 : c + 1;
            if (live && tm.valid(m) && MHD_SM(pb + c * 3, 12) && MHD_SM(pb + cp * 3, 4) &&
                MHD_GM(bjp + c * 3 + 1, a.b, MHD_NB(f)) && MHD_GM(bkp + c * 3 + 2, a.b, MHD_NB(f))) {
                bc[m][0] = fadd(0.5f * pb[c * 3 + 0], 0.5f * pb[cp * 3 + 0]);
                bc[m][1] = fadd(0.5f * pb[c * 3 + 1], 0.5f * bjp[c * 3 + 1]);
                bc[m][2] = fadd(0.5f * pb[c * 3 + 2], 0.5f * bkp[c * 3 + 2]);
            } else {
                bc[m][0] = 0.0f; bc[m][1] = 0.0f; bc[m][2] = 0.0f;
            }
        }
    } else {
        const long long kb = (long long)k * f.sk;
        const int kp = (k + 1 == f.nz) ? 0 : k + 1;
        const long long kpb = (long long)kp * f.sk;
        const int bs = fx_bs(n);
        const int ks = ppc + 1;                          // SK row stride (odd for ppc = 2^m)
        float *SB = XA;                                  // (ppc+1) * bs: frame b of columns j0..j0+nvalid
        float *SK = XA + (size_t)(ppc + 1) * bs;         // n * ks: frame b(3) of plane k+1, [i][q]
        const int ru = 5 * nvalid, rb = 3 * (nvalid + 1);
        const int pb2 = nib(f.pb, 2);
        // Per-lane offsets do not depend on the row: a row of u is ru floats
        // at u_in + (rowc + j0)*5, element r -> pencil r/5, component r%5.
        // (ru <= 40, rb <= 27 for ppc <= 8: at most two elements per lane.)
        int us_off[2], sb_off[2], gb_off[2];
        bool us_on[2], sb_on[2];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int r = lane + 32 * h;
            us_on[h] = r < ru;
            const int qq = r / 5, p = r - qq * 5;
            us_off[h] = qq * ps + nib(f.iu, p);
            sb_on[h] = r < rb;
            const int qb = r / 3, pp = r - qb * 3;
            int j = j0 + qb;
            if (j >= f.ny) j -= f.ny;
            sb_off[h] = qb * bs + nib(f.ib, pp);
            gb_off[h] = j * 3 + pp;
        }
        const bool sk_on = lane < nvalid;
        for (int i = warp; i < n; i += nwarps) {
            const long long rowc = kb + (long long)i * f.si;    // cell of (i, 0, k)
            const float *gu = a.u_in + (rowc + j0) * 5;
            const float *gb = a.b + rowc * 3;
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                if (us_on[h] && MHD_GM(gu + lane + 32 * h, a.u_in, MHD_NU(f)))
                    cp_async4(&US[us_off[h] + i * 5], gu + lane + 32 * h);
                if (sb_on[h] && MHD_GM(gb + gb_off[h], a.b, MHD_NB(f))) cp_async4(&SB[sb_off[h] + i * 3], gb + gb_off[h]);
            }
            const float *gk = a.b + (kpb + (long long)i * f.si + j0 + lane) * 3 + pb2;
            if (sk_on && MHD_GM(gk, a.b, MHD_NB(f))) cp_async4(&SK[i * ks + lane], gk);
        }
        cp_async_wait_all();
        __syncthreads();
        const float *sb0 = SB + (size_t)q * bs, *sb1 = SB + (size_t)(q + 1) * bs;
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            const int c = tm.ci(m);
            const int cp = (c + 1 == n) ? 0 : c + 1;
            if (live && tm.valid(m) && MHD_SM(sb0 + c * 3, 12) && MHD_SM(sb0 + cp * 3, 4) &&
                MHD_SM(sb1 + c * 3 + 1, 4) && MHD_SM(&SK[c * ks + q], 4)) {
                bc[m][0] = fadd(0.5f * sb0[c * 3 + 0], 0.5f * sb0[cp * 3 + 0]);
                bc[m][1] = fadd(0.5f * sb0[c * 3 + 1], 0.5f * sb1[c * 3 + 1]);
                bc[m][2] = fadd(0.5f * sb0[c * 3 + 2], 0.5f * SK[c * ks + q]);
            } else {
                bc[m][0] = 0.0f; bc[m][1] = 0.0f; bc[m][2] = 0.0f;
            }
        }
    }
    __syncthreads();   // the exchange area of one pencil overlaps the staged b of others

    const float hdt = 0.5f * dt;
    unsigned bad = 0;
    float u1[CPL][5];

    // ================= half step =================
    // rows 0-4: wl = u - v/c ; rows 5-9: flux
    {
        float v[CPL][5];
        float cl = 0.0f;
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            if (!tm.valid(m)) continue;   // padding slots compute nothing
            float uu[5];
            if (live) {
#pragma unroll
                for (int ii = 0; ii < 5; ++ii) uu[ii] = UR(tm.ci(m) * 5 + ii);
            } else {
                uu[0] = 1.0f; uu[1] = 0.0f; uu[2] = 0.0f; uu[3] = 0.0f; uu[4] = 1.0f;
            }
            float cs, p;
            cell_flux<M>(uu, bc[m], v[m], cs, p);
            cl = fmaxf(cl, cs);
        }
        const float c = tm.pencil_max(cl, rq);
        // v/c where c > 0 (mhdflux.c:48-57); where c = 0 the quotient by 1
        // leaves every finite v as it is, without a select per value
        const float cd = c > 0.0f ? c : 1.0f;
        const float yc = M::recip(cd);
        // fr = c(u + v/c) kept in u1[]; wl exchanged
#pragma unroll
        for (int m = 0; m < CPL; ++m)
#pragma unroll
            for (int ii = 0; ii < 5; ++ii) if (tm.valid(m)) {
                const float uu = UR(tm.ci(m) * 5 + ii);
                const float vv = M::divy(v[m][ii], cd, yc);
                u1[m][ii] = M::mul(c, M::add(uu, vv));
                tm.put(X(ii), m, M::sub(uu, vv));
            }
        tm.sync();
        // flux = (fr - c*cshift(wl,+1))/2
#pragma unroll
        for (int m = 0; m < CPL; ++m)
#pragma unroll
            for (int ii = 0; ii < 5; ++ii) if (tm.valid(m)) {
                const float fl = M::mul(c, XR(ii, tm.ci(m) + 1));
                u1[m][ii] = 0.5f * M::sub(u1[m][ii], fl);
                tm.put(X(5 + ii), m, u1[m][ii]);
            }
        tm.sync();
        // u1 = u - (flux - cshift(flux,-1)) dt/2
#pragma unroll
        for (int m = 0; m < CPL; ++m)
#pragma unroll
            for (int ii = 0; ii < 5; ++ii) if (tm.valid(m)) {
                const float d = M::sub(u1[m][ii], XR(5 + ii, tm.ci(m) - 1));
                u1[m][ii] = M::add(UR(tm.ci(m) * 5 + ii), M::mul(-hdt, d));
            }
    }
    tm.sync();   // every read of rows 5-9 is done before they are rewritten

    // ================= full step =================
    // rows 0-4: fr, then the flux ; rows 5-9: wl
    {
        float cl = 0.0f;
        {
            float v[CPL][5];
#pragma unroll
            for (int m = 0; m < CPL; ++m) {
                if (!tm.valid(m)) continue;
                float cs, p;
                cell_flux<M>(u1[m], bc[m], v[m], cs, p);
                cl = fmaxf(cl, cs);
                if (!(p > 0.0f)) bad |= MHD_HEALTH_PRESSURE;
            }
            const float c = tm.pencil_max(cl, rq);
            cl = c;
            // v/c where c > 0 (mhdflux.c:48-57); where c = 0 the quotient by 1
            // leaves every finite v as it is, without a select per value
            const float cd = c > 0.0f ? c : 1.0f;
            const float yc = M::recip(cd);
#pragma unroll
            for (int m = 0; m < CPL; ++m)
#pragma unroll
                for (int ii = 0; ii < 5; ++ii) if (tm.valid(m)) {
                    const float vv = M::divy(v[m][ii], cd, yc);
                    tm.put(X(ii), m, M::mul(c, M::add(u1[m][ii], vv)));
                    tm.put(X(5 + ii), m, M::sub(u1[m][ii], vv));
                }
        }
        const float c = cl;
        tm.sync();
        // flux = (fr - fl + dfr - dfl)/2 with van Leer slopes (tvd1.c:54-112);
        // fl(i) = c wl(i+1), fl(i+1) = c wl(i+2), fl(i-1) = c wl(i).  The
        // limiter inputs are the undivided differences (the reference's /2
        // factors cancel exactly in 2ab/(a+b)).
        float fx[CPL][5];
#pragma unroll
        for (int m = 0; m < CPL; ++m)
#pragma unroll
            for (int ii = 0; ii < 5; ++ii) if (tm.valid(m)) {
                const int cm = tm.ci(m);
                const float f0 = XR(ii, cm);
                const float dfr = M::slope(M::sub(XR(ii, cm + 1), f0), M::sub(f0, XR(ii, cm - 1)));
                const float fl0 = M::mul(c, XR(5 + ii, cm + 1));
                const float flp = M::mul(c, XR(5 + ii, cm + 2));
                const float flm = M::mul(c, XR(5 + ii, cm));
                const float dfl = M::slope(M::sub(fl0, flp), M::sub(flm, fl0));
                fx[m][ii] = 0.5f * M::add(M::sub(f0, fl0), M::sub(dfr, dfl));
            }
        tm.sync();
#pragma unroll
        for (int m = 0; m < CPL; ++m)
#pragma unroll
            for (int ii = 0; ii < 5; ++ii) tm.put(X(ii), m, fx[m][ii]);
        tm.sync();
        // u = u - (flux - cshift(flux,-1)) dt, written back into US
        const float mdt = -dt;
        const bool fold_cfl = !ROWS && a.cfl != nullptr;
        const float *bown = a.b + (p0 + q) * 3 * n;   // !ROWS: this pencil's b
        float cfl_c = 0.0f;
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            if (!(live && tm.valid(m))) continue;
            const int cc = tm.ci(m);
            float s = 0.0f, r = 0.0f;
            float uf[5];
#pragma unroll
            for (int ii = 0; ii < 5; ++ii) {
                const float d = M::sub(fx[m][ii], XR(ii, cc - 1));
                const float un = M::add(UR(cc * 5 + ii), M::mul(mdt, d));
                if (MHD_SM(us + cc * 5 + ii, 4)) us[cc * 5 + ii] = un;
                uf[ii] = un;
                s += un;
                if (ii == 0) r = un;
            }
            if (!(r > 0.0f)) bad |= MHD_HEALTH_DENSITY;
            if (!isfinite(s)) bad |= MHD_HEALTH_NONFINITE;
            if (fold_cfl) {
                // the CFL fast speed of the updated cell, as cfl_cell_speed forms it
                float bb[3];
                if (!(MHD_GM(bown + cc * 3, a.b, MHD_NB(f)) && MHD_GM(bown + cc * 3 + 2, a.b, MHD_NB(f)) &&
                      MHD_GM(bown + ((cc + 1 == n) ? 0 : cc + 1) * 3, a.b, MHD_NB(f)) &&
                      MHD_GM(bjp + cc * 3 + 1, a.b, MHD_NB(f)) &&
                      MHD_GM(bkp + cc * 3 + 2, a.b, MHD_NB(f))))
                    continue;
                if (a.cfl_mode == MHD_CFL_C) {
                    bb[0] = bown[cc * 3 + 0];
                    bb[1] = bown[cc * 3 + 1];
                    bb[2] = bown[cc * 3 + 2];
                    cfl_c = fmaxf(cfl_c, cfl_speed_c(uf, bb));
                } else {
                    const int cp = (cc + 1 == n) ? 0 : cc + 1;
                    bb[0] = fdiv(fadd(bown[cc * 3 + 0], bown[cp * 3 + 0]), 2.0f);
                    bb[1] = fdiv(fadd(bown[cc * 3 + 1], bjp[cc * 3 + 1]), 2.0f);
                    bb[2] = fdiv(fadd(bown[cc * 3 + 2], bkp[cc * 3 + 2]), 2.0f);
                    cfl_c = fmaxf(cfl_c, cfl_speed_averaged(uf, bb));
                }
            }
        }
        if (fold_cfl) cfl_warp_max(cfl_c, a.cfl);   // every lane of the warp
    }

    if (!live) bad = 0;
    if (bad) flag_health(a.health, bad);
    __syncthreads();
    if (!ROWS) {
        if (MHD_GM(a.u_out + p0 * 5 * n, a.u_out, MHD_NU(f)) &&
            MHD_GM(a.u_out + (p0 + nvalid) * 5 * n - 1, a.u_out, MHD_NU(f)))
            block_copy_out(a.u_out + p0 * 5 * n, US, (long long)nvalid * 5 * n, threadIdx.x, blockDim.x);
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
            off[h] = qq * ps + nib(f.iu, p);
        }
        for (int i = warp; i < n; i += nwarps) {
            float *g = a.u_out + (kb + (long long)i * f.si + j0) * 5;
#pragma unroll
            for (int h = 0; h < 2; ++h)
                if (on[h] && MHD_SM(&US[off[h] + i * 5], 4) && MHD_GM(g + lane + 32 * h, a.u_out, MHD_NU(f)))
                    g[lane + 32 * h] = US[off[h] + i * 5];
        }
    }
}

// One CTA's work on a tile; called once per CTA by fluidx_kernel and in a loop
// by the batched kernel (batch_kernel.cuh).  Pencils that fill a team of at
// most one warp exactly take the register-blocked tile (same results;
// FLAGGED: its flagged pass, see fluidx_tile_reg).
template <int CPL, int WPP, class M, bool ROWS, int NT, bool GROUPED = false, bool FLAGGED = false>
__device__ __forceinline__ void fluidx_tile(const FluidxArgs &a, long long tile)
{
    if constexpr (NT > 0 && reg_tile_shape(NT, CPL, WPP))
        fluidx_tile_reg<CPL, team_threads<WPP>(), M, ROWS, GROUPED, false, FLAGGED>(a, tile);
    else
        fluidx_tile_team<CPL, WPP, M, ROWS, NT>(a, tile);
}

template <int CPL, int WPP, class M, bool ROWS, int NT>
__global__ void __launch_bounds__(256)
fluidx_kernel(const __grid_constant__ FluidxArgs a)
{
    fluidx_tile<CPL, WPP, M, ROWS, NT, true>(a, blockIdx.x);
}

// The row-staged sweep with its tile moved by TMA (tma_rows.cuh): pencils
// that fill one warp (NT = 32 CPL), kTmaPencils per CTA, in place.
template <int CPL, class M, int NT>
__global__ void __launch_bounds__(32 * kTmaPencils)
fluidx_kernel_tma(const __grid_constant__ FluidxArgs a, const __grid_constant__ RowMaps maps)
{
    fluidx_tile_reg<CPL, 32, M, true, true, true>(a, blockIdx.x, &maps);
}

// Launch one instantiation; sets the dynamic shared-memory attribute once per
// instantiation when above the 48 KB default.
template <int CPL, int WPP, class M, bool ROWS, int NT>
cudaError_t launch_fluidx_inst(const FluidxArgs &a, int ppc, cudaStream_t s)
{
    if constexpr (ROWS && WPP == 1 && NT == 32 * CPL) {
        // row-staged pencils that fill a warp: through TMA when the frame allows
        RowMaps maps;
        if (row_staging() == MHD_STAGING_TMA && ppc == kTmaPencils && a.u_out == a.u_in &&
            tma_rows_encode(&maps, a.u_in, a.b, a.f.n, a.f.ny, a.f.nz, a.f.si, a.f.sk, kTmaPencils)) {
            static std::atomic<size_t> smem_tma[kSmemCacheDevices];
            const size_t smem = sizeof(float) * (size_t)txr_smem_floats(fxr_smem_floats(NT, ppc, true), NT);
            if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
            const cudaError_t e =
                ensure_dynamic_smem((const void *)fluidx_kernel_tma<CPL, M, NT>, smem, smem_tma);
            if (e != cudaSuccess) return e;
            const long long blocks = (long long)((a.f.ny + ppc - 1) / ppc) * a.f.nz;
            fluidx_kernel_tma<CPL, M, NT><<<(unsigned)blocks, 32 * ppc, smem, s>>>(a, maps);
            return cudaGetLastError();
        }
    }
    static std::atomic<size_t> smem_set[kSmemCacheDevices];
    const int threads = 32 * WPP * ppc;
    const long long blocks = ROWS ? (long long)((a.f.ny + ppc - 1) / ppc) * a.f.nz
                                  : (a.f.npen + ppc - 1) / ppc;
    const size_t smem = sizeof(float) * (size_t)fx_tile_smem_floats(NT > 0 ? NT : a.f.n, ppc, CPL, WPP, ROWS);
    if (smem > 227 * 1024) return cudaErrorInvalidConfiguration;
    const cudaError_t e = ensure_dynamic_smem((const void *)fluidx_kernel<CPL, WPP, M, ROWS, NT>, smem, smem_set);
    if (e != cudaSuccess) return e;
    fluidx_kernel<CPL, WPP, M, ROWS, NT><<<(unsigned)blocks, threads, smem, s>>>(a);
    return cudaGetLastError();
}

// dispatch over the supported team shapes, both staging modes (rows mode
// when the frame's pencils run across memory, frame_rows) and the
// compile-time length when the pencil fills the team exactly
template <int C, int W, class M>
cudaError_t launch_fluidx_shape(const FluidxArgs &a, int ppc, bool rows, cudaStream_t s)
{
    constexpr int CAP = 32 * W * C;
    if (a.f.n == CAP)
        return rows ? launch_fluidx_inst<C, W, M, true, CAP>(a, ppc, s)
                    : launch_fluidx_inst<C, W, M, false, CAP>(a, ppc, s);
    return rows ? launch_fluidx_inst<C, W, M, true, 0>(a, ppc, s)
                : launch_fluidx_inst<C, W, M, false, 0>(a, ppc, s);
}

template <class M>
cudaError_t launch_fluidx_policy(const FluidxArgs &a, const PencilCfg &cfg, cudaStream_t s)
{
    const bool rows = frame_rows(a.f);
#define MHD_FX(C, W) \
    if (cfg.cpl == C && cfg.wpp == W) return launch_fluidx_shape<C, W, M>(a, cfg.ppc, rows, s);
    MHD_PENCIL_SHAPES(MHD_FX)
#undef MHD_FX
    return cudaErrorInvalidConfiguration;
}

}  // namespace mhd
