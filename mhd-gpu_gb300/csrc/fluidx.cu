// fluidx.cu - the fluid sweep (relaxing TVD, RK2) on pencils of the reference
// layout, for sm_103a.
//
// Algorithm: Heterogeneous_MHD/C/fluidx.c:19-102 (gather + cell-centred B),
// tvd1.c:8-118 (RK2 half and full step, van Leer limiter), mhdflux.c:9-72
// (flux vector and pencil-wide max fast speed).
//
// GB300 mapping.  A CTA owns PPC consecutive pencils p = j + ny*k, so its u
// and b inputs are each one contiguous chunk (5n and 3n floats per pencil):
// they are staged into shared memory with 16-byte coalesced loads, and the
// result leaves the same way.  Each pencil belongs to a team of 32*WPP
// threads that keeps CPL cells per thread in registers for the whole update.
// The stencil neighbours (i-1, i+1, i+2) are exchanged through a per-pencil
// shared-memory buffer, and the two pencil-wide maxima of the fast speed are
// warp-shuffle reductions (plus one shared-memory step when WPP > 1).
// Nothing is a contraction, so there are no tensor cores here: the kernel is
// bounded by FP32 issue and HBM bandwidth.
#include "kernels.cuh"

namespace mhd {

// shared floats per pencil: stage/exchange region X1 (10n) + X2 (5n)
__host__ __device__ constexpr int fluidx_smem_floats_per_pencil(int n) { return 15 * n; }

template <int CPL, int WPP>
__global__ void __launch_bounds__(256)
fluidx_kernel(FluidxArgs a)
{
    constexpr int TPP = 32 * WPP;
    extern __shared__ float smem[];
    const int n = a.f.n;
    const int ppc = blockDim.x / TPP;
    const int q = threadIdx.x / TPP;
    const long long p0 = (long long)blockIdx.x * ppc;
    const long long pen = p0 + q;
    const int nvalid = (int)min((long long)ppc, a.f.npen - p0);
    const bool live = q < nvalid;

    float *X1 = smem;                       // ppc * 10n
    float *X2 = smem + (size_t)ppc * 10 * n; // ppc * 5n
    float *red = X2 + (size_t)ppc * 5 * n;   // ppc * WPP
    float *x1 = X1 + (size_t)q * 10 * n;
    float *x2 = X2 + (size_t)q * 5 * n;
    float *rq = red + q * WPP;

    Team<CPL, WPP> tm;
    tm.init(threadIdx.x - q * TPP, n);
    const float dt = *a.dt;

    // ---- stage u and own b chunks (contiguous) ----
    float *su = X1;                              // nvalid*5n
    float *sb = X1 + (size_t)ppc * 5 * n;        // nvalid*3n
    block_copy_in(su, a.u_in + p0 * 5 * n, (long long)nvalid * 5 * n, threadIdx.x, blockDim.x);
    block_copy_in(sb, a.b + p0 * 3 * n, (long long)nvalid * 3 * n, threadIdx.x, blockDim.x);
    __syncthreads();

    float u[CPL][5], bc[CPL][3];
    {
        const int j = live ? (int)(pen % a.f.ny) : 0;
        const int k = live ? (int)(pen / a.f.ny) : 0;
        const int jp = (j + 1 == a.f.ny) ? 0 : j + 1;
        const int kp = (k + 1 == a.f.nz) ? 0 : k + 1;
        const float *bjp = a.b + ((long long)k * a.f.ny + jp) * 3 * n;
        const float *bkp = a.b + ((long long)kp * a.f.ny + j) * 3 * n;
        const float *pu = su + (size_t)q * 5 * n;
        const float *pb = sb + (size_t)q * 3 * n;
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            const int c = tm.cell[m];
            if (live && tm.valid[m]) {
#pragma unroll
                for (int ii = 0; ii < 5; ++ii) u[m][ii] = pu[c * 5 + ii];
                // b3x = b/2 ; b3x(1) += cshift(b3x(1),1) ; b3x(2) += b(2,jp)/2 ;
                // b3x(3) += b(3,kp)/2   (fluidx.c:71-81; the halvings are exact)
                bc[m][0] = fadd(0.5f * pb[c * 3 + 0], 0.5f * pb[tm.ip[m] * 3 + 0]);
                bc[m][1] = fadd(0.5f * pb[c * 3 + 1], 0.5f * bjp[c * 3 + 1]);
                bc[m][2] = fadd(0.5f * pb[c * 3 + 2], 0.5f * bkp[c * 3 + 2]);
            } else {
                u[m][0] = 1.0f; u[m][1] = 0.0f; u[m][2] = 0.0f; u[m][3] = 0.0f; u[m][4] = 1.0f;
                bc[m][0] = 0.0f; bc[m][1] = 0.0f; bc[m][2] = 0.0f;
            }
        }
    }
    __syncthreads();   // X1 of one pencil overlaps the staged chunk of others

    const float hdt = 0.5f * dt;
    float u1[CPL][5];
    unsigned bad = 0;

    // ================= half step =================
    {
        float v[CPL][5];
        float cl = 0.0f;
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            float cs, p;
            cell_flux(u[m], bc[m], v[m], cs, p);
            if (tm.valid[m]) cl = fmaxf(cl, cs);
        }
        const float c = tm.pencil_max(cl, rq);
        if (c > 0.0f) {
#pragma unroll
            for (int m = 0; m < CPL; ++m)
#pragma unroll
                for (int ii = 0; ii < 5; ++ii) v[m][ii] = fdiv(v[m][ii], c);
        }
        // fr = c(u+v) kept; wl = u-v exchanged
        float fr[CPL][5];
#pragma unroll
        for (int m = 0; m < CPL; ++m)
#pragma unroll
            for (int ii = 0; ii < 5; ++ii) {
                fr[m][ii] = fmul(c, fadd(u[m][ii], v[m][ii]));
                if (tm.valid[m]) x1[ii * n + tm.cell[m]] = fsub(u[m][ii], v[m][ii]);
            }
        tm.sync();
        // flux = (fr - c*cshift(wl,+1))/2
        float fx[CPL][5];
#pragma unroll
        for (int m = 0; m < CPL; ++m)
#pragma unroll
            for (int ii = 0; ii < 5; ++ii) {
                const float fl = fmul(c, x1[ii * n + tm.ip[m]]);
                fx[m][ii] = 0.5f * fsub(fr[m][ii], fl);
                if (tm.valid[m]) x2[ii * n + tm.cell[m]] = fx[m][ii];
            }
        tm.sync();
        // u1 = u - (flux - cshift(flux,-1)) dt/2
#pragma unroll
        for (int m = 0; m < CPL; ++m)
#pragma unroll
            for (int ii = 0; ii < 5; ++ii) {
                const float d = fsub(fx[m][ii], x2[ii * n + tm.im[m]]);
                u1[m][ii] = fadd(u[m][ii], fmul(-hdt, d));
            }
    }

    // ================= full step =================
    {
        float v[CPL][5];
        float cl = 0.0f;
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            float cs, p;
            cell_flux(u1[m], bc[m], v[m], cs, p);
            if (tm.valid[m]) {
                cl = fmaxf(cl, cs);
                if (!(p > 0.0f)) bad |= MHD_HEALTH_PRESSURE;
            }
        }
        const float c = tm.pencil_max(cl, rq);
        if (c > 0.0f) {
#pragma unroll
            for (int m = 0; m < CPL; ++m)
#pragma unroll
                for (int ii = 0; ii < 5; ++ii) v[m][ii] = fdiv(v[m][ii], c);
        }
        // exchange fr = c(u1+v) and wl = u1-v
        float fr[CPL][5];
#pragma unroll
        for (int m = 0; m < CPL; ++m)
#pragma unroll
            for (int ii = 0; ii < 5; ++ii) {
                fr[m][ii] = fmul(c, fadd(u1[m][ii], v[m][ii]));
                if (tm.valid[m]) {
                    x1[ii * n + tm.cell[m]] = fr[m][ii];
                    x1[(5 + ii) * n + tm.cell[m]] = fsub(u1[m][ii], v[m][ii]);
                }
            }
        tm.sync();
        float fx[CPL][5];
#pragma unroll
        for (int m = 0; m < CPL; ++m)
#pragma unroll
            for (int ii = 0; ii < 5; ++ii) {
                const float f0 = fr[m][ii];
                const float frp = x1[ii * n + tm.ip[m]];
                const float frm = x1[ii * n + tm.im[m]];
                const float dfr = van_leer(0.5f * fsub(frp, f0), 0.5f * fsub(f0, frm));
                // fl = c*cshift(wl,+1): fl(i) = c wl(i+1), fl(i+1) = c wl(i+2), fl(i-1) = c wl(i)
                const float fl0 = fmul(c, x1[(5 + ii) * n + tm.ip[m]]);
                const float flp = fmul(c, x1[(5 + ii) * n + tm.ipp[m]]);
                const float flm = fmul(c, x1[(5 + ii) * n + tm.cell[m]]);
                const float dfl = van_leer(0.5f * fsub(fl0, flp), 0.5f * fsub(flm, fl0));
                fx[m][ii] = 0.5f * fadd(fsub(f0, fl0), fsub(dfr, dfl));
                if (tm.valid[m]) x2[ii * n + tm.cell[m]] = fx[m][ii];
            }
        tm.sync();
        const float mdt = -dt;
#pragma unroll
        for (int m = 0; m < CPL; ++m)
#pragma unroll
            for (int ii = 0; ii < 5; ++ii) {
                const float d = fsub(fx[m][ii], x2[ii * n + tm.im[m]]);
                u[m][ii] = fadd(u[m][ii], fmul(mdt, d));
            }
    }

    // ---- health and store through the staging buffer ----
    __syncthreads();   // every team is done reading X1/X2
    {
        float *pu = X1 + (size_t)q * 5 * n;
#pragma unroll
        for (int m = 0; m < CPL; ++m) {
            if (live && tm.valid[m]) {
                const int c = tm.cell[m];
                float s = 0.0f;
#pragma unroll
                for (int ii = 0; ii < 5; ++ii) { pu[c * 5 + ii] = u[m][ii]; s += u[m][ii]; }
                if (!(u[m][0] > 0.0f)) bad |= MHD_HEALTH_DENSITY;
                if (!isfinite(s)) bad |= MHD_HEALTH_NONFINITE;
            }
        }
    }
    if (!live) bad = 0;
    if (bad) flag_health(a.health, bad);
    __syncthreads();
    block_copy_out(a.u_out + p0 * 5 * n, X1, (long long)nvalid * 5 * n, threadIdx.x, blockDim.x);
}

// ---------------------------------------------------------------------------
// launch table: (CPL, WPP) by pencil length.  The team covers n <= 32*WPP*CPL.
// ---------------------------------------------------------------------------
PencilCfg fluidx_pick(int n)
{
    if (n <= 32)  return {1, 1, 8};
    if (n <= 64)  return {2, 1, 4};
    if (n <= 128) return {4, 1, 4};
    if (n <= 256) return {4, 2, 2};
    if (n <= 512) return {4, 4, 1};
    return {4, 8, 1};
}

cudaError_t launch_fluidx(const FluidxArgs &a, const PencilCfg &cfg, cudaStream_t s)
{
    const int tpp = 32 * cfg.wpp;
    const int threads = tpp * cfg.ppc;
    const long long blocks = (a.f.npen + cfg.ppc - 1) / cfg.ppc;
    const size_t smem = sizeof(float) * ((size_t)cfg.ppc * fluidx_smem_floats_per_pencil(a.f.n)
                                         + (size_t)cfg.ppc * cfg.wpp);
#define MHD_FLUIDX_CASE(C, W)                                                                  \
    if (cfg.cpl == C && cfg.wpp == W) {                                                        \
        static int smem_set_##C##_##W = 0;                                                     \
        if (smem > 48 * 1024 && (size_t)smem_set_##C##_##W < smem) {                           \
            cudaError_t e = cudaFuncSetAttribute(fluidx_kernel<C, W>,                          \
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                                 (int)smem);                                   \
            if (e != cudaSuccess) return e;                                                    \
            smem_set_##C##_##W = (int)smem;                                                    \
        }                                                                                      \
        fluidx_kernel<C, W><<<(unsigned)blocks, threads, smem, s>>>(a);                        \
        return cudaGetLastError();                                                             \
    }
    MHD_FLUIDX_CASE(1, 1)
    MHD_FLUIDX_CASE(2, 1)
    MHD_FLUIDX_CASE(4, 1)
    MHD_FLUIDX_CASE(4, 2)
    MHD_FLUIDX_CASE(4, 4)
    MHD_FLUIDX_CASE(4, 8)
#undef MHD_FLUIDX_CASE
    return cudaErrorInvalidConfiguration;
}

}  // namespace mhd
