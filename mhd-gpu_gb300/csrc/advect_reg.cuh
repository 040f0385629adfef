// advect_reg.cuh - the field advection (advectbyzx flux pass), register-blocked,
// for pencils whose length fills a team of at most one warp exactly (the 32,
// 48, 64, 96 and 128-cell pencils).
//
// Algorithm and rounding: exactly advect_tile's (advect_kernel.cuh; reference
// Heterogeneous_MHD/C/advectbyzxA1.c:18-63, B1.c:19-62, tvdb.c:10-91),
// operation for operation, so the two give the same bits.  As in
// fluidx_reg.cuh, thread t of a team owns the cells t*CPL .. t*CPL+CPL-1 and
// takes stencil neighbours from its registers or the adjacent lanes (warp
// shuffles); the two stages (A: frame b(2) with the velocity averaged with
// the j-1 pencil, B: b(3) with the k-1 pencil) run one after the other on the
// same registers.  Inputs are staged per pencil as runs of n cells (rho and m
// of the own, j-1 and k-1 pencils, own b(2) and b(3)), outputs (b(2), b(3),
// sA, sB) go back through the same area so that the global writes are
// coalesced in either staging mode.
#pragma once

#include <type_traits>

#include "fluidx_reg.cuh"

#undef MHD_DBG_FILE
#define MHD_DBG_FILE 3

namespace mhd {

// shared floats: 8 arrays of ppc runs of n+4 floats (16-byte aligned runs)
__host__ __device__ inline int axr_run(int n) { return n + 4; }
__host__ __device__ inline long long axr_smem_floats(int n, int ppc) { return 8LL * ppc * axr_run(n); }

// arrays of the staging area
enum { kAxRho = 0, kAxM = 1, kAxRhoJ = 2, kAxMJ = 3, kAxRhoK = 4, kAxMK = 5, kAxB2 = 6, kAxB3 = 7 };

template <int CPL, int TPP, bool ROWS, class MP>
__device__ __forceinline__ bool advect_tile_reg_pass(const AdvectArgs &a, long long tile, MP &mp)
{
    constexpr int N = TPP * CPL, R = N + 4;
    extern __shared__ __align__(16) float smem_r[];
    float *smem = smem_r;
    const Frame &f = a.f;
    const int ppc = blockDim.x / TPP;
    const int q = threadIdx.x / TPP;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const Lanes<TPP> ln{(int)(threadIdx.x & (TPP - 1))};
    const int c0 = ln.t * CPL;
    const int PR = ppc * R;   // one array

    long long pen = 0;         // !ROWS: this team's pencil
    int j0 = 0, k = 0, nvalid;
    if (!ROWS) {
        const long long p0 = tile * ppc;
        nvalid = (int)min((long long)ppc, f.npen - p0);
        pen = p0 + q;
    } else {
        const int njb = (f.ny + ppc - 1) / ppc;
        k = (int)(tile / njb);
        j0 = (int)(tile - (long long)k * njb) * ppc;
        nvalid = min(ppc, f.ny - j0);
    }
    const bool live = q < nvalid;

    // ---- stage the inputs ----
    if (!ROWS) {
        // each team stages its own pencil's runs, lanes on consecutive cells
        if (live) {
            const unsigned kk = fast_div((unsigned)pen, a.dny);
            const int j = (int)((unsigned)pen - kk * (unsigned)f.ny);
            const long long pjm = (j == 0) ? pen + f.ny - 1 : pen - 1;
            const long long pkm = (kk == 0) ? pen + (long long)(f.nz - 1) * f.ny : pen - f.ny;
            const float *uo = a.u + pen * N * 5, *uj = a.u + pjm * N * 5, *uk = a.u + pkm * N * 5;
            const float *bo = a.b + pen * N * 3;
            float *d = smem + q * R;
#pragma unroll
            for (int s = 0; s < CPL; ++s) {
                const int c = ln.t + s * TPP;
                if (!(MHD_GM(uo + c * 5 + 1, a.u, MHD_NU(f)) && MHD_GM(uj + c * 5 + 1, a.u, MHD_NU(f)) &&
                      MHD_GM(uk + c * 5 + 1, a.u, MHD_NU(f)) && MHD_GM(bo + c * 3 + 2, a.b, MHD_NB(f))))
                    continue;
                cp_async4(d + kAxRho * PR + c, uo + c * 5);
                cp_async4(d + kAxM * PR + c, uo + c * 5 + 1);
                cp_async4(d + kAxRhoJ * PR + c, uj + c * 5);
                cp_async4(d + kAxMJ * PR + c, uj + c * 5 + 1);
                cp_async4(d + kAxRhoK * PR + c, uk + c * 5);
                cp_async4(d + kAxMK * PR + c, uk + c * 5 + 1);
                cp_async4(d + kAxB2 * PR + c, bo + c * 3 + 1);
                cp_async4(d + kAxB3 * PR + c, bo + c * 3 + 2);
            }
        }
    } else {
        // row i of the tile: one value per (array, pencil); lane L = array*ppc +
        // pencil, so consecutive lanes read neighbouring cells of one row
        const int km = (k == 0) ? f.nz - 1 : k - 1;
        const int pm = nib(f.pu, 1), p2 = nib(f.pb, 1), p3 = nib(f.pb, 2);
        const float *src[2];
        long long gst[2];
        int dst[2];
        bool on[2];
#if defined(MHD_DEBUG)
        const float *glo[2];
        long long gn[2];
#endif
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int L = lane + 32 * h;
            const int arr = L / ppc, qq = L - arr * ppc;
            on[h] = arr < 8 && qq < nvalid;
            const bool isb = arr >= kAxB2;
            int jc = j0 + qq - ((arr == kAxRhoJ || arr == kAxMJ) ? 1 : 0);
            if (jc < 0) jc += f.ny;
            const int plane = (arr == kAxRhoK || arr == kAxMK) ? km : k;
            const int comp = isb ? (arr == kAxB2 ? p2 : p3) : ((arr & 1) ? pm : 0);
            const long long cell = (long long)plane * f.sk + jc;
            src[h] = isb ? a.b + cell * 3 + comp : a.u + cell * 5 + comp;
            gst[h] = (isb ? 3 : 5) * f.si;
#if defined(MHD_DEBUG)
            glo[h] = isb ? a.b : a.u;
            gn[h] = isb ? MHD_NB(f) : MHD_NU(f);
#endif
            dst[h] = on[h] ? arr * PR + qq * R : 0;
        }
        for (int i = warp; i < N; i += nwarps) {
#pragma unroll
            for (int h = 0; h < 2; ++h)
                if (on[h] && MHD_GM(src[h] + (long long)i * gst[h], glo[h], gn[h]))
                    cp_async4(smem + dst[h] + i, src[h] + (long long)i * gst[h]);
        }
    }
    cp_async_wait_all();
    __syncthreads();

    const float dt = *a.dt;
    float bout[2][CPL], sout[2][CPL];
    const float *run = smem + q * R + c0;   // this thread's cells in array 0
#pragma unroll
    for (int st = 0; st < 2; ++st) {
        // vx = (m(nb) + m)/(rho(nb) + rho), nb = the j-1 (A) or k-1 (B) pencil
        // (A1.c:58, B1.c:51); the stage's own field component
        float v[CPL], bb[CPL];
        if (live) {
            float ro[CPL], mo[CPL], rn[CPL], mn[CPL];
            lds_run<CPL>(run + kAxRho * PR, ro);
            lds_run<CPL>(run + kAxM * PR, mo);
            lds_run<CPL>(run + (st ? kAxRhoK : kAxRhoJ) * PR, rn);
            lds_run<CPL>(run + (st ? kAxMK : kAxMJ) * PR, mn);
            lds_run<CPL>(run + (st ? kAxB3 : kAxB2) * PR, bb);
#pragma unroll
            for (int m = 0; m < CPL; ++m) v[m] = mp.div(mp.add(mn[m], mo[m]), mp.add(rn[m], ro[m]));
        } else {
#pragma unroll
            for (int m = 0; m < CPL; ++m) { v[m] = 0.0f; bb[m] = 0.0f; }
        }
        // vg = (cshift(v,-1) + cshift(v,1) + 2 v)/4: the (s + 2v)/4 is formed in
        // double by the reference and rounded once; the quarter is exact
        const float vl = ln.from(v[CPL - 1], -1), vr = ln.from(v[0], 1);
        float g[CPL], bg[CPL];
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            const float s = mp.add(m > 0 ? v[m - 1] : vl, m + 1 < CPL ? v[m + 1] : vr);
            g[m] = 0.25f * mp.twice_plus(v[m], s);
            bg[m] = mp.mul(bb[m], g[m]);
        }
        // tvdb: vh = (vg + cshift(vg,1))/2 ; flux1 = b vg, upwinded by vh
        const float gr = ln.from(g[0], 1), bgr = ln.from(bg[0], 1);
        float h[CPL], f1[CPL];
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            h[m] = mp.add(0.5f * g[m], 0.5f * (m + 1 < CPL ? g[m + 1] : gr));
            f1[m] = (h[m] > 0.0f) ? bg[m] : (m + 1 < CPL ? bg[m + 1] : bgr);
        }
        // b1 = b - (flux1 - cshift(flux1,-1)) dt/2 (the product float, the
        // halving and the subtraction double in the reference: one rounding)
        const float f1l = ln.from(f1[CPL - 1], -1);
        float gb[CPL];
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            const float b1 = mp.minus_half(bb[m], mp.mul(mp.sub(f1[m], m > 0 ? f1[m - 1] : f1l), dt));
            gb[m] = mp.mul(g[m], b1);
        }
        // upwind second-order flux on the right face with the van Leer limiter
        // (tvdb.c:64-75), from vg*b1 of cells c-1 .. c+2
        const float gbl = ln.from(gb[CPL - 1], -1), gbr1 = ln.from(gb[0], 1);
        const float gbr2 = (CPL >= 2) ? ln.from(gb[CPL >= 2 ? 1 : 0], 1) : ln.from(gb[0], 2);
        auto GB = [&](int i) { return i < 0 ? gbl : (i < CPL ? gb[i] : (i == CPL ? gbr1 : gbr2)); };
        float fl[CPL];
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            const bool up = h[m] > 0.0f;
            const float w = up ? GB(m) : GB(m + 1);
            const float Wp = up ? mp.sub(GB(m + 1), w) : mp.sub(w, GB(m + 2));
            const float Wm = up ? mp.sub(w, GB(m - 1)) : mp.sub(GB(m), w);
            const float dw = mp.slope(Wm, Wp);
            fl[m] = mp.mul(mp.add(w, dw), dt);
        }
        // b = b - (flux - cshift(flux,-1)) ; the shifted flux is kept for b(1)
        const float fll = ln.from(fl[CPL - 1], -1);
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            const float sp = m > 0 ? fl[m - 1] : fll;
            bout[st][m] = mp.sub(bb[m], mp.sub(fl[m], sp));
            sout[st][m] = sp;
        }
    }

    // A flagged pass writes nothing when a lane of the CTA formed a value near
    // a rounding boundary: its caller computes the tile again exactly.
    if constexpr (MP::kFlagged) {
        if (__syncthreads_or(mp.nb ? 1 : 0)) return false;
    }
    // ---- outputs through shared memory: arrays b(2), b(3), sA, sB ----
    __syncthreads();   // the inputs are consumed
    if (live) {
        float *o = smem + q * R + c0;
        sts_run<CPL>(o, bout[0]);
        sts_run<CPL>(o + PR, bout[1]);
        sts_run<CPL>(o + 2 * PR, sout[0]);
        sts_run<CPL>(o + 3 * PR, sout[1]);
    }
    __syncthreads();
    const int p2 = nib(f.pb, 1), p3 = nib(f.pb, 2);
    if (!ROWS) {
        if (live) {
            const float *o = smem + q * R;
            float *gb = a.b + pen * N * 3;
            float *ga = a.sA + pen * N, *gs = a.sB + pen * N;
#pragma unroll
            for (int s = 0; s < CPL; ++s) {
                const int c = ln.t + s * TPP;
                if (!(MHD_SM(&o[c], 4) && MHD_SM(&o[3 * PR + c], 4) && MHD_GM(gb + c * 3 + 2, a.b, MHD_NB(f)) &&
                      MHD_GM(ga + c, a.sA, f.npen * f.n) && MHD_GM(gs + c, a.sB, f.npen * f.n)))
                    continue;
                gb[c * 3 + p2] = o[c];
                gb[c * 3 + p3] = o[PR + c];
                ga[c] = o[2 * PR + c];
                gs[c] = o[3 * PR + c];
            }
        }
    } else {
        // row i: lane L = array*ppc + pencil (4*ppc <= 32 lanes); each lane's
        // destination array and stride chosen once
        const long long kb = (long long)k * f.sk;
        const int w = lane / ppc, qq = lane - w * ppc;
        const bool on = w < 4 && qq < nvalid;
        float *const dst = w == 0 ? a.b + p2 : (w == 1 ? a.b + p3 : (w == 2 ? a.sA : a.sB));
        const int dstride = w < 2 ? 3 : 1;
        const float *o = smem + (on ? w * PR + qq * R : 0);
        for (int i = warp; i < N; i += nwarps) {
            if (!on) continue;
            const long long cell = kb + (long long)i * f.si + j0 + qq;
            if (MHD_SM(&o[i], 4) && MHD_GM(dst + cell * dstride, w < 2 ? a.b : (w == 2 ? a.sA : a.sB),
                                           w < 2 ? MHD_NB(f) : f.npen * f.n))
                dst[cell * dstride] = o[i];
        }
    }
    return true;
}

// the exact pass of a flagged tile, after the flagged pass (see
// fluidx_tile_reg_exact)
template <int CPL, int TPP, bool ROWS>
__device__ __forceinline__ void advect_tile_reg_exact(const AdvectArgs &a, long long tile)
{
    Faithful m;
    advect_tile_reg_pass<CPL, TPP, ROWS>(a, tile, m);
}

// One tile of the field sweep; FLAGGED (the batched kernels): Faithful runs
// as FaithfulNB first (see fluidx_tile_reg).
template <int CPL, int TPP, class M, bool ROWS, bool FLAGGED = false>
__device__ __forceinline__ void advect_tile_reg(const AdvectArgs &a, long long tile)
{
    if constexpr (FLAGGED && std::is_same<M, Faithful>::value) {
        FaithfulNB f;
        if (!advect_tile_reg_pass<CPL, TPP, ROWS>(a, tile, f)) {
            __syncthreads();   // the flagged pass's shared memory is consumed
            advect_tile_reg_exact<CPL, TPP, ROWS>(a, tile);
        }
    } else {
        M m;
        advect_tile_reg_pass<CPL, TPP, ROWS>(a, tile, m);
    }
}

}  // namespace mhd
