// advect_kernel.cuh - constrained-transport advection of the transverse face fields
// (advectbyzx) on pencils of a frame view, for sm_103a.
//
// Algorithm: Heterogeneous_MHD/C/advectbyzx.c:14-23 with advectbyzxA1.c:18-63,
// A2.c:9-28, B1.c:19-62, B2.c:9-29 and the upwind/van Leer 1-D update tvdb.c:10-91.
//
// The reference scatters b(1)(j-1) += flux(j) through a full-grid temporary in
// a second pass.  Here:
//   kernel 1 (per pencil team, like fluidx) advects frame b(2) (stage A,
//     velocity averaged with the j-1 pencil) and b(3) (stage B, with the k-1
//     pencil) in the same pass, writes them in place, and writes the shifted
//     fluxes sA(i,j,k) = fluxA(i-1,j,k), sB(i,j,k) = fluxB(i-1,j,k) to scratch
//     indexed like the stored cells;
//   kernel 2 (one thread per stored cell) gathers
//     b(1) = (((b(1) - sA(j)) + sA(j+1)) - sB(k)) + sB(k+1),
//   which is the reference's per-cell rounding order (A1, A2, B1, B2).
// Stage B reads only the pre-advection b(3) and u, so fusing A and B in one
// kernel changes no value.  Pencils that run across memory (the y and z
// sweeps of an x-major box) are staged through shared memory in rows, as in
// fluidx_kernel.cuh.  Pencils of 32, 48, 64, 96 or 128 cells take the
// register-blocked tile of advect_reg.cuh, every other length the team tile
// below (same arithmetic).
#pragma once

#include "advect_reg.cuh"
#include "kernels.cuh"

#undef MHD_DBG_FILE
#define MHD_DBG_FILE 4

namespace mhd {

// shared floats: two alternating exchange buffers of 4 per cell and pencil,
// plus, for pencils across memory, the row staging (rho and m of the j-1
// column and the k-1 plane, own b(2) b(3); reused for the outputs)
// Row staging layouts are [i][column] with odd row strides, so a warp reading
// one column down consecutive cells hits 32 different banks.
__host__ __device__ inline int ax_r2(int ppc) { return 2 * (ppc + 1) + 1; }   // U2 row
__host__ __device__ inline int ax_rk(int ppc) { return 2 * ppc + 1; }         // UK, BO row
__host__ __device__ inline int ax_ro(int ppc) { return 4 * ppc + 1; }         // output row
// exchange area of one pencil: 8 halo rows of n+3 floats (two alternating
// groups of four)
__host__ __device__ inline long long ax_xpen(int n) { return 8LL * (n + 3); }
__host__ __device__ inline long long ax_smem_floats(int n, int ppc, bool rows)
{
    long long s = ax_xpen(n) * ppc;
    if (rows) s += (long long)n * (ax_r2(ppc) + 2 * ax_rk(ppc));
    return s;
}
// shared floats of the tile that a (cpl, wpp) team takes for pencils of n
// cells: register-blocked (advect_reg.cuh) when the pencil fills the team
__host__ __device__ inline long long ax_tile_smem_floats(int n, int ppc, int cpl, int wpp, bool rows)
{
    return reg_tile_shape(n, cpl, wpp) ? axr_smem_floats(n, ppc) : ax_smem_floats(n, ppc, rows);
}

// One CTA's work on its group of pencils (see fluidx_tile_team), any pencil
// length up to the team's capacity.
template <int CPL, int WPP, class M, bool ROWS, int NT>
__device__ __forceinline__ void advect_tile_team(const AdvectArgs &a, long long tile)
{
    constexpr int TPP = team_threads<WPP>();
    extern __shared__ float smem[];
    const Frame &f = a.f;
    const int n = NT > 0 ? NT : f.n;
    const int ppc = blockDim.x / TPP;
    const int q = threadIdx.x / TPP;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;

    long long pen = 0;
    int j0 = 0, k = 0, nvalid = 0;
    if (!ROWS) {
        pen = tile * ppc + q;
    } else {
        const int njb = (f.ny + ppc - 1) / ppc;
        k = (int)(tile / njb);
        j0 = (int)(tile - (long long)k * njb) * ppc;
        nvalid = min(ppc, f.ny - j0);
    }
    const bool live = ROWS ? q < nvalid : pen < f.npen;
    float *ST = smem + (size_t)ppc * ax_xpen(n);

    Team<CPL, WPP, NT> tm;
    tm.init(threadIdx.x - q * TPP, n);
    const float dt = *a.dt;
    const int rs = tm.rs();
    float *xbase = smem + (size_t)q * ax_xpen(n) + 1;
    auto X = [&](int r) { return xbase + r * rs; };
    // value of exchange row r at cell i (-1 <= i <= n+1)
    auto XR = [&](int r, int i) { return (MHD_IN(i + 1, rs) && MHD_SM(X(r) + i, 4)) ? X(r)[i] : 0.0f; };

    float vA[CPL], vB[CPL], bA[CPL], bB[CPL];
    long long base = 0;   // !ROWS: first stored cell of the pencil
    if (!ROWS) {
        const int j = live ? (int)(pen % f.ny) : 0;
        const int kk = live ? (int)(pen / f.ny) : 0;
        const int jm = (j == 0) ? f.ny - 1 : j - 1;
        const int km = (kk == 0) ? f.nz - 1 : kk - 1;
        base = ((long long)kk * f.ny + j) * n;
        const long long bjm = ((long long)kk * f.ny + jm) * n;
        const long long bkm = ((long long)km * f.ny + j) * n;
        // vx = (m_x(jm) + m_x) / (rho(jm) + rho)  (A1.c:58, B1.c:51)
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            const int c = tm.ci(m);
            if (live && tm.valid(m) && MHD_GM(a.u + (base + c) * 5 + 1, a.u, MHD_NU(f)) &&
                MHD_GM(a.u + (bjm + c) * 5 + 1, a.u, MHD_NU(f)) && MHD_GM(a.u + (bkm + c) * 5 + 1, a.u, MHD_NU(f)) &&
                MHD_GM(a.b + (base + c) * 3 + 2, a.b, MHD_NB(f))) {
                const float r0 = a.u[(base + c) * 5 + 0], m0 = a.u[(base + c) * 5 + 1];
                const float rj = a.u[(bjm + c) * 5 + 0], mj = a.u[(bjm + c) * 5 + 1];
                const float rk = a.u[(bkm + c) * 5 + 0], mk = a.u[(bkm + c) * 5 + 1];
                vA[m] = M::div(M::add(mj, m0), M::add(rj, r0));
                vB[m] = M::div(M::add(mk, m0), M::add(rk, r0));
                bA[m] = a.b[(base + c) * 3 + 1];
                bB[m] = a.b[(base + c) * 3 + 2];
            } else {
                vA[m] = 0.0f; vB[m] = 0.0f; bA[m] = 0.0f; bB[m] = 0.0f;
            }
        }
    } else {
        // rows of the tile: U2 = (rho, m) of columns j0-1 .. j0+nvalid-1 at k,
        // UK = (rho, m) of columns j0 .. at k-1, BO = own (b(2), b(3))
        float *U2 = ST;
        const int r2 = ax_r2(ppc), rk = ax_rk(ppc);
        float *UK = U2 + (size_t)n * r2;                  // n * rk
        float *BO = UK + (size_t)n * rk;                  // n * rk
        const int km = (k == 0) ? f.nz - 1 : k - 1;
        const long long kb = (long long)k * f.sk, kmb = (long long)km * f.sk;
        const int pm = nib(f.pu, 1), p2 = nib(f.pb, 1), p3 = nib(f.pb, 2);
        // per-lane column offsets (2*(ppc+1) <= 18 columns for ppc <= 8)
        const int qq = lane >> 1, w = lane & 1;
        const bool on2 = lane < 2 * (nvalid + 1), onk = lane < 2 * nvalid;
        int jc = j0 - 1 + qq;
        if (jc < 0) jc += f.ny;
        if (jc >= f.ny) jc -= f.ny;
        const int g2 = jc * 5 + (w ? pm : 0);
        const int gk = (j0 + qq) * 5 + (w ? pm : 0);
        const int gb = (j0 + qq) * 3 + (w ? p3 : p2);
        for (int i = warp; i < n; i += nwarps) {
            const long long rowc = kb + (long long)i * f.si;
            const long long rowk = kmb + (long long)i * f.si;
            if (on2 && MHD_GM(a.u + rowc * 5 + g2, a.u, MHD_NU(f))) cp_async4(&U2[i * r2 + lane], a.u + rowc * 5 + g2);
            if (onk && MHD_GM(a.u + rowk * 5 + gk, a.u, MHD_NU(f)) && MHD_GM(a.b + rowc * 3 + gb, a.b, MHD_NB(f))) {
                cp_async4(&UK[i * rk + lane], a.u + rowk * 5 + gk);
                cp_async4(&BO[i * rk + lane], a.b + rowc * 3 + gb);
            }
        }
        cp_async_wait_all();
        __syncthreads();
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            const int c = tm.ci(m);
            const float *uo = U2 + c * r2 + 2 * (q + 1), *uj = U2 + c * r2 + 2 * q;
            const float *uk = UK + c * rk + 2 * q, *bo = BO + c * rk + 2 * q;
            if (live && tm.valid(m) && MHD_SM(uo, 8) && MHD_SM(uj, 8) && MHD_SM(uk, 8) && MHD_SM(bo, 8)) {
                vA[m] = M::div(M::add(uj[1], uo[1]), M::add(uj[0], uo[0]));
                vB[m] = M::div(M::add(uk[1], uo[1]), M::add(uk[0], uo[0]));
                bA[m] = bo[0];
                bB[m] = bo[1];
            } else {
                vA[m] = 0.0f; vB[m] = 0.0f; bA[m] = 0.0f; bB[m] = 0.0f;
            }
        }
    }
    // rows 0,1 <- the face velocities
#pragma unroll
    for (int m = 0; m < CPL; ++m) { tm.put(X(0), m, vA[m]); tm.put(X(1), m, vB[m]); }
    tm.sync();
    // vx = (cshift(vx,-1) + cshift(vx,1) + 2 vx)/4: the (s + 2vx)/4 is formed
    // in double by the reference and rounded once; the quarter is exact.
    // rows 4-7 <- vg and b*vg of both stages
    float gA[CPL], gB[CPL];   // smoothed velocities vg
#pragma unroll
    for (int m = 0; m < CPL; ++m) {
        if (!tm.valid(m)) continue;   // padding slots compute nothing
        const int c = tm.ci(m);
        const float sa = M::add(XR(0, c - 1), XR(0, c + 1));
        const float sb = M::add(XR(1, c - 1), XR(1, c + 1));
        gA[m] = 0.25f * M::twice_plus(vA[m], sa);
        gB[m] = 0.25f * M::twice_plus(vB[m], sb);
        tm.put(X(4), m, gA[m]);
        tm.put(X(5), m, gB[m]);
        tm.put(X(6), m, M::mul(bA[m], gA[m]));
        tm.put(X(7), m, M::mul(bB[m], gB[m]));
    }
    tm.sync();
    // tvdb: vh = (vg + cshift(vg,1))/2 ; flux1 = b vg, upwinded by vh ; rows 0,1 <- flux1
    float hA[CPL], hB[CPL], f1A[CPL], f1B[CPL];
#pragma unroll
    for (int m = 0; m < CPL; ++m) {
        if (!tm.valid(m)) continue;
        const int c = tm.ci(m);
        hA[m] = M::add(0.5f * gA[m], 0.5f * XR(4, c + 1));
        hB[m] = M::add(0.5f * gB[m], 0.5f * XR(5, c + 1));
        f1A[m] = (hA[m] > 0.0f) ? XR(6, c) : XR(6, c + 1);
        f1B[m] = (hB[m] > 0.0f) ? XR(7, c) : XR(7, c + 1);
        tm.put(X(0), m, f1A[m]);
        tm.put(X(1), m, f1B[m]);
    }
    tm.sync();
    // b1 = b - (flux1 - cshift(flux1,-1)) dt/2 : the product is float, the
    // halving and the subtraction double in the reference -> one rounding.
    // rows 4,5 <- vg*b1
#pragma unroll
    for (int m = 0; m < CPL; ++m) {
        if (!tm.valid(m)) continue;
        const int c = tm.ci(m);
        const float b1A = M::minus_half(bA[m], M::mul(M::sub(f1A[m], XR(0, c - 1)), dt));
        const float b1B = M::minus_half(bB[m], M::mul(M::sub(f1B[m], XR(1, c - 1)), dt));
        tm.put(X(4), m, M::mul(gA[m], b1A));
        tm.put(X(5), m, M::mul(gB[m], b1B));
    }
    tm.sync();
    // upwind second-order flux on the right face with the van Leer limiter;
    // wp, wm are half differences, so the slope of the undivided ones is
    // 2 wm wp/(wm+wp) exactly (tvdb.c:64-75) ; rows 2,3 <- flux
    float flA[CPL], flB[CPL];
#pragma unroll
    for (int m = 0; m < CPL; ++m) {
        if (!tm.valid(m)) continue;
        const int c = tm.ci(m);
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const float h = s ? hB[m] : hA[m];
            float w, Wp, Wm;
            if (h > 0.0f) {
                w = XR(4 + s, c);
                Wp = M::sub(XR(4 + s, c + 1), w);
                Wm = M::sub(w, XR(4 + s, c - 1));
            } else {
                w = XR(4 + s, c + 1);
                Wp = M::sub(w, XR(4 + s, c + 2));
                Wm = M::sub(XR(4 + s, c), w);
            }
            const float dw = M::slope(Wm, Wp);
            const float fl = M::mul(M::add(w, dw), dt);
            if (s) flB[m] = fl; else flA[m] = fl;
        }
        tm.put(X(2), m, flA[m]);
        tm.put(X(3), m, flB[m]);
    }
    tm.sync();
    // b = b - (flux - cshift(flux,-1)) ; outputs b(2), b(3), sA, sB
    if (!ROWS) {
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            if (live && tm.valid(m) && MHD_GM(a.b + (base + tm.ci(m)) * 3 + 2, a.b, MHD_NB(f)) &&
                MHD_GM(a.sA + base + tm.ci(m), a.sA, f.npen * n) && MHD_GM(a.sB + base + tm.ci(m), a.sB, f.npen * n)) {
                const int c = tm.ci(m);
                const float sa = XR(2, c - 1), sb = XR(3, c - 1);
                a.b[(base + c) * 3 + 1] = M::sub(bA[m], M::sub(flA[m], sa));
                a.b[(base + c) * 3 + 2] = M::sub(bB[m], M::sub(flB[m], sb));
                a.sA[base + c] = sa;
                a.sB[base + c] = sb;
            }
        }
    } else {
        float o[CPL][4];
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            if (!tm.valid(m)) continue;
            const int c = tm.ci(m);
            const float sa = XR(2, c - 1), sb = XR(3, c - 1);
            o[m][0] = M::sub(bA[m], M::sub(flA[m], sa));
            o[m][1] = M::sub(bB[m], M::sub(flB[m], sb));
            o[m][2] = sa;
            o[m][3] = sb;
        }
        const int ro = ax_ro(ppc);
        float *OUT = ST;   // n * ro: row i holds (b(2), b(3), sA, sB) of each pencil
        __syncthreads();   // the row staging is consumed
#pragma unroll
        for (int m = 0; m < CPL; ++m)
            if (live && tm.valid(m))
#pragma unroll
                for (int w = 0; w < 4; ++w)
                    if (MHD_SM(&OUT[tm.ci(m) * ro + 4 * q + w], 4)) OUT[tm.ci(m) * ro + 4 * q + w] = o[m][w];
        __syncthreads();
        const long long kb = (long long)k * f.sk;
        const int p2 = nib(f.pb, 1), p3 = nib(f.pb, 2);
        const int qq = lane >> 2, w = lane & 3;      // 4*ppc <= 32 values per row
        const bool on = lane < 4 * nvalid;
        // each lane's destination array and stride, chosen once (no divergent
        // stores in the loop)
        float *const dst = w == 0 ? a.b + p2 : (w == 1 ? a.b + p3 : (w == 2 ? a.sA : a.sB));
        const int dstride = w < 2 ? 3 : 1;
        for (int i = warp; i < n; i += nwarps) {
            if (!on) continue;
            const long long cell = kb + (long long)i * f.si + j0 + qq;
            if (MHD_SM(&OUT[i * ro + lane], 4) && MHD_GM(dst + cell * dstride, w < 2 ? a.b : (w == 2 ? a.sA : a.sB),
                                                          w < 2 ? MHD_NB(f) : f.npen * n))
                dst[cell * dstride] = OUT[i * ro + lane];
        }
    }
}

// One CTA's work on a tile (advect_flux_kernel, the batched kernel): pencils
// that fill a team of at most one warp exactly take the register-blocked tile
// (same results; FLAGGED: its flagged pass, see fluidx_tile_reg).
template <int CPL, int WPP, class M, bool ROWS, int NT, bool FLAGGED = false>
__device__ __forceinline__ void advect_tile(const AdvectArgs &a, long long tile)
{
    if constexpr (NT > 0 && reg_tile_shape(NT, CPL, WPP))
        advect_tile_reg<CPL, team_threads<WPP>(), M, ROWS, FLAGGED>(a, tile);
    else
        advect_tile_team<CPL, WPP, M, ROWS, NT>(a, tile);
}

// b(1) = (((b(1) - sA(i,j,k)) + sA(i,j+1,k)) - sB(i,j,k)) + sB(i,j,k+1) for
// stored cell c; j, k and the neighbours follow the frame's strides.  Plain
// coherent loads: the batched sweep kernel writes sA, sB earlier in the same
// launch.  (ncell < 2^31: the index arithmetic runs in 32 bits, the divisions
// as multiplies, FastDiv.)
// the j+1 and k+1 neighbours of stored cell c in the frame (periodic)
__device__ __forceinline__ void advect_b1_neighbours(const AdvectArgs &a, unsigned c, unsigned &cj, unsigned &ck)
{
    const Frame &f = a.f;
    const unsigned qj = fast_div(c, a.dsj), qk = fast_div(c, a.dsk);
    const unsigned j = qj - fast_div(qj, a.dny) * (unsigned)f.ny;
    const unsigned k = qk - fast_div(qk, a.dnz) * (unsigned)f.nz;
    const unsigned sj = (unsigned)f.sj, sk = (unsigned)f.sk;
    cj = (j + 1 == (unsigned)f.ny) ? c - j * sj : c + sj;
    ck = (k + 1 == (unsigned)f.nz) ? c - k * sk : c + sk;
}

__device__ __forceinline__ void advect_b1_cell(const AdvectArgs &a, unsigned c)
{
    const Frame &f = a.f;
    unsigned cj, ck;
    advect_b1_neighbours(a, c, cj, ck);
    const int p1 = nib(f.pb, 0);
    const long long ncell = f.npen * f.n;
    (void)ncell;
    if (!(MHD_IN(c, ncell) && MHD_IN(cj, ncell) && MHD_IN(ck, ncell))) return;
    float *bp = a.b + (size_t)c * 3 + p1;
    float bx = *bp;
    bx = fsub(bx, a.sA[c]);
    bx = fadd(bx, a.sA[cj]);
    bx = fsub(bx, a.sB[c]);
    bx = fadd(bx, a.sB[ck]);
    *bp = bx;
}

// G cells c, c + step, .. at once: every load of the G is issued before the
// first store, so a thread has 5 G loads in flight (the stores go to b, which
// the compiler cannot tell apart from the flux arrays).  Same arithmetic per
// cell as advect_b1_cell.
template <int G>
__device__ __forceinline__ void advect_b1_cells(const AdvectArgs &a, unsigned c, unsigned step)
{
    const Frame &f = a.f;
    const int p1 = nib(f.pb, 0);
    const long long ncell = f.npen * f.n;
    (void)ncell;
    float v[G][5];
    float *bp[G];
    bool ok[G];
#pragma unroll
    for (int k = 0; k < G; ++k) {
        const unsigned ck0 = c + k * step;
        unsigned cj, ck;
        advect_b1_neighbours(a, ck0, cj, ck);
        ok[k] = MHD_IN(ck0, ncell) && MHD_IN(cj, ncell) && MHD_IN(ck, ncell);
        bp[k] = a.b + (size_t)ck0 * 3 + p1;
        if (ok[k]) {
            v[k][0] = *bp[k];
            v[k][1] = a.sA[ck0];
            v[k][2] = a.sA[cj];
            v[k][3] = a.sB[ck0];
            v[k][4] = a.sB[ck];
        }
    }
#pragma unroll
    for (int k = 0; k < G; ++k) {
        if (!ok[k]) continue;
        float bx = fsub(v[k][0], v[k][1]);
        bx = fadd(bx, v[k][2]);
        bx = fsub(bx, v[k][3]);
        bx = fadd(bx, v[k][4]);
        *bp[k] = bx;
    }
}

}  // namespace mhd
