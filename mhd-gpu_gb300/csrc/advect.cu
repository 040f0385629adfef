// advect.cu - constrained-transport advection of the transverse face fields
// (advectbyzx) on pencils of the reference layout, for sm_103a.
//
// Algorithm: Heterogeneous_MHD/C/advectbyzx.c:14-23 with advectbyzxA1.c:18-63,
// A2.c:9-28, B1.c:19-62, B2.c:9-29 and the upwind/van Leer 1-D update tvdb.c:10-91.
//
// The reference scatters b_x(j-1) += flux(j) through a full-grid temporary in
// a second pass.  Here:
//   kernel 1 (per pencil team, like fluidx) advects b_y (stage A, velocity
//     averaged with the j-1 pencil) and b_z (stage B, with the k-1 pencil) in
//     the same pass, writes them in place, and writes the shifted fluxes
//     sA(i,j,k) = fluxA(i-1,j,k), sB(i,j,k) = fluxB(i-1,j,k) to caller scratch;
//   kernel 2 (one thread per cell) gathers
//     b_x = (((b_x - sA(j)) + sA(j+1)) - sB(k)) + sB(k+1),
//   which is the reference's per-cell rounding order (A1, A2, B1, B2).
// Stage B reads only the pre-advection b_z and u, so fusing A and B in one
// kernel changes no value.
#include "kernels.cuh"

namespace mhd {

// one exchange buffer holds 4 floats per cell; two alternate
__host__ __device__ constexpr int advect_smem_floats_per_pencil(int n) { return 8 * n; }

template <int CPL, int WPP>
__global__ void __launch_bounds__(256)
advect_flux_kernel(AdvectArgs a)
{
    constexpr int TPP = 32 * WPP;
    extern __shared__ float smem[];
    const int n = a.f.n;
    const int ppc = blockDim.x / TPP;
    const int q = threadIdx.x / TPP;
    const long long pen = (long long)blockIdx.x * ppc + q;
    const bool live = pen < a.f.npen;
    float *xa = smem + (size_t)q * 8 * n;  // buffer 0
    float *xb = xa + 4 * n;                // buffer 1

    Team<CPL, WPP> tm;
    tm.init(threadIdx.x - q * TPP, n);
    const float dt = *a.dt;

    const int j = live ? (int)(pen % a.f.ny) : 0;
    const int k = live ? (int)(pen / a.f.ny) : 0;
    const int jm = (j == 0) ? a.f.ny - 1 : j - 1;
    const int km = (k == 0) ? a.f.nz - 1 : k - 1;
    const long long base = ((long long)k * a.f.ny + j) * n;
    const long long bjm = ((long long)k * a.f.ny + jm) * n;
    const long long bkm = ((long long)km * a.f.ny + j) * n;

    // ---- per-cell velocity at the j-1/2 (A) and k-1/2 (B) faces ----
    float vA[CPL], vB[CPL], bA[CPL], bB[CPL];
#pragma unroll
    for (int m = 0; m < CPL; ++m) {
        const int c = tm.cell[m];
        if (live && tm.valid[m]) {
            const float r0 = a.u[(base + c) * 5 + 0], m0 = a.u[(base + c) * 5 + 1];
            const float rj = a.u[(bjm + c) * 5 + 0], mj = a.u[(bjm + c) * 5 + 1];
            const float rk = a.u[(bkm + c) * 5 + 0], mk = a.u[(bkm + c) * 5 + 1];
            vA[m] = fdiv(fadd(mj, m0), fadd(rj, r0));
            vB[m] = fdiv(fadd(mk, m0), fadd(rk, r0));
            bA[m] = a.b[(base + c) * 3 + 1];
            bB[m] = a.b[(base + c) * 3 + 2];
        } else {
            vA[m] = 0.0f; vB[m] = 0.0f; bA[m] = 0.0f; bB[m] = 0.0f;
        }
        if (tm.valid[m]) { xa[c] = vA[m]; xa[n + c] = vB[m]; }
    }
    tm.sync();
    // vx = (cshift(vx,-1) + cshift(vx,1) + 2 vx)/4 ; the (s + 2vx)/4 is formed
    // in double by the reference and rounded once: fma + exact quarter.
    float gA[CPL], gB[CPL];   // smoothed velocities vg
#pragma unroll
    for (int m = 0; m < CPL; ++m) {
        const float sa = fadd(xa[tm.im[m]], xa[tm.ip[m]]);
        const float sb = fadd(xa[n + tm.im[m]], xa[n + tm.ip[m]]);
        gA[m] = 0.25f * ffma(2.0f, vA[m], sa);
        gB[m] = 0.25f * ffma(2.0f, vB[m], sb);
        if (tm.valid[m]) {
            const int c = tm.cell[m];
            xb[c] = gA[m]; xb[n + c] = gB[m];
            xb[2 * n + c] = fmul(bA[m], gA[m]);
            xb[3 * n + c] = fmul(bB[m], gB[m]);
        }
    }
    tm.sync();
    // tvdb: vh = (vg + cshift(vg,1))/2 ; flux1 = b vg (upwind by vh)
    float hA[CPL], hB[CPL], f1A[CPL], f1B[CPL];
#pragma unroll
    for (int m = 0; m < CPL; ++m) {
        const int c = tm.cell[m], cp = tm.ip[m];
        hA[m] = fadd(0.5f * gA[m], 0.5f * xb[cp]);
        hB[m] = fadd(0.5f * gB[m], 0.5f * xb[n + cp]);
        f1A[m] = (hA[m] > 0.0f) ? xb[2 * n + c] : xb[2 * n + cp];
        f1B[m] = (hB[m] > 0.0f) ? xb[3 * n + c] : xb[3 * n + cp];
        if (tm.valid[m]) { xa[c] = f1A[m]; xa[n + c] = f1B[m]; }
    }
    tm.sync();
    // b1 = b - (flux1 - cshift(flux1,-1)) dt/2 : the product is float, the
    // halving and the subtraction are double in the reference -> one rounding.
    // Then exchange the products vg*b1.
#pragma unroll
    for (int m = 0; m < CPL; ++m) {
        const int cm = tm.im[m];
        const float b1A = ffma(-0.5f, fmul(fsub(f1A[m], xa[cm]), dt), bA[m]);
        const float b1B = ffma(-0.5f, fmul(fsub(f1B[m], xa[n + cm]), dt), bB[m]);
        if (tm.valid[m]) {
            const int c = tm.cell[m];
            xb[c] = fmul(gA[m], b1A);
            xb[n + c] = fmul(gB[m], b1B);
        }
    }
    tm.sync();
    // upwind second-order flux on the right face with van Leer limiting
    float flA[CPL], flB[CPL];
#pragma unroll
    for (int m = 0; m < CPL; ++m) {
        const int c = tm.cell[m], cp = tm.ip[m], cpp = tm.ipp[m], cm = tm.im[m];
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const float *g = xb + s * n;
            const float h = s ? hB[m] : hA[m];
            float w, wp, wm;
            if (h > 0.0f) {
                w = g[c];
                wp = 0.5f * fsub(g[cp], w);
                wm = 0.5f * fsub(w, g[cm]);
            } else {
                w = g[cp];
                wp = 0.5f * fsub(w, g[cpp]);
                wm = 0.5f * fsub(g[c], w);
            }
            const float dw = van_leer(wm, wp);
            const float fl = fmul(fadd(w, dw), dt);
            if (s) flB[m] = fl; else flA[m] = fl;
        }
        if (tm.valid[m]) { xa[2 * n + c] = flA[m]; xa[3 * n + c] = flB[m]; }
    }
    tm.sync();
    // b = b - (flux - cshift(flux,-1)) ; store b_y, b_z and the shifted flux
#pragma unroll
    for (int m = 0; m < CPL; ++m) {
        if (live && tm.valid[m]) {
            const int c = tm.cell[m], cm = tm.im[m];
            const float sa = xa[2 * n + cm], sb = xa[3 * n + cm];
            a.b[(base + c) * 3 + 1] = fsub(bA[m], fsub(flA[m], sa));
            a.b[(base + c) * 3 + 2] = fsub(bB[m], fsub(flB[m], sb));
            a.sA[base + c] = sa;
            a.sB[base + c] = sb;
        }
    }
}

// b_x(i,j,k) = (((b_x - sA(i,j,k)) + sA(i,j+1,k)) - sB(i,j,k)) + sB(i,j,k+1)
__global__ void __launch_bounds__(256)
advect_bx_kernel(float *__restrict__ b, const float *__restrict__ sA, const float *__restrict__ sB,
                 Frame f, long long ncell)
{
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    const long long pen = c / f.n;
    const int i = (int)(c - pen * f.n);
    const int j = (int)(pen % f.ny);
    const int k = (int)(pen / f.ny);
    const int jp = (j + 1 == f.ny) ? 0 : j + 1;
    const int kp = (k + 1 == f.nz) ? 0 : k + 1;
    const long long cj = ((long long)k * f.ny + jp) * f.n + i;
    const long long ck = ((long long)kp * f.ny + j) * f.n + i;
    float bx = b[c * 3];
    bx = fsub(bx, sA[c]);
    bx = fadd(bx, sA[cj]);
    bx = fsub(bx, sB[c]);
    bx = fadd(bx, sB[ck]);
    b[c * 3] = bx;
}

PencilCfg advect_pick(int n)
{
    if (n <= 32)  return {1, 1, 8};
    if (n <= 64)  return {2, 1, 4};
    if (n <= 128) return {4, 1, 4};
    if (n <= 256) return {4, 2, 2};
    if (n <= 512) return {4, 4, 1};
    return {4, 8, 1};
}

cudaError_t launch_advect(const AdvectArgs &a, const PencilCfg &cfg, cudaStream_t s)
{
    const int tpp = 32 * cfg.wpp;
    const int threads = tpp * cfg.ppc;
    const long long blocks = (a.f.npen + cfg.ppc - 1) / cfg.ppc;
    const size_t smem = sizeof(float) * (size_t)cfg.ppc * advect_smem_floats_per_pencil(a.f.n);
    cudaError_t e = cudaErrorInvalidConfiguration;
#define MHD_ADVECT_CASE(C, W)                                                                  \
    if (cfg.cpl == C && cfg.wpp == W) {                                                        \
        static int smem_set_##C##_##W = 0;                                                     \
        if (smem > 48 * 1024 && (size_t)smem_set_##C##_##W < smem) {                           \
            e = cudaFuncSetAttribute(advect_flux_kernel<C, W>,                                 \
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);  \
            if (e != cudaSuccess) return e;                                                    \
            smem_set_##C##_##W = (int)smem;                                                    \
        }                                                                                      \
        advect_flux_kernel<C, W><<<(unsigned)blocks, threads, smem, s>>>(a);                   \
        e = cudaGetLastError();                                                                \
    }
    MHD_ADVECT_CASE(1, 1)
    else MHD_ADVECT_CASE(2, 1)
    else MHD_ADVECT_CASE(4, 1)
    else MHD_ADVECT_CASE(4, 2)
    else MHD_ADVECT_CASE(4, 4)
    else MHD_ADVECT_CASE(4, 8)
#undef MHD_ADVECT_CASE
    if (e != cudaSuccess) return e;
    const long long ncell = a.f.npen * a.f.n;
    const long long nb = (ncell + 255) / 256;
    advect_bx_kernel<<<(unsigned)nb, 256, 0, s>>>(a.b, a.sA, a.sB, a.f, ncell);
    return cudaGetLastError();
}

}  // namespace mhd
