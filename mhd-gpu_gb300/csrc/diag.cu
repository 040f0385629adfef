// diag.cu - FP64 diagnostics of a state on the device (mhdgpu_diagnostics):
// totals of mass, momentum and energy, max |div B| of the face field, and the
// gas pressure's minimum and count of non-positive cells.
//
// The reference prints float sums of the state from the host after a run
// (Heterogeneous_MHD/C/check_value.c:22-79); at 512^3 a float sum of 1.3e8
// terms loses every digit below ~1e-1 relative, so here every term and every
// partial sum is a double.  The reduction order is fixed by the box size
// (grid-stride pass with a fixed grid, then one block in block order), so the
// result is reproducible run to run.
#include "kernels.cuh"

namespace mhd {

constexpr int kDiagThreads = 256;
constexpr int kDiagBlocksMax = 152 * 4;

struct DiagAcc {
    double s[5];      // rho, m_x, m_y, m_z, E
    double divb;      // max |div B|
    double pmin;      // min p
    double nneg;      // cells with p <= 0
};

__device__ __forceinline__ void diag_merge(DiagAcc &a, const DiagAcc &b)
{
#pragma unroll
    for (int i = 0; i < 5; ++i) a.s[i] += b.s[i];
    a.divb = fmax(a.divb, b.divb);
    a.pmin = fmin(a.pmin, b.pmin);
    a.nneg += b.nneg;
}

__device__ __forceinline__ void diag_shfl(DiagAcc &a, int o)
{
    DiagAcc b;
#pragma unroll
    for (int i = 0; i < 5; ++i) b.s[i] = __shfl_down_sync(0xffffffffu, a.s[i], o);
    b.divb = __shfl_down_sync(0xffffffffu, a.divb, o);
    b.pmin = __shfl_down_sync(0xffffffffu, a.pmin, o);
    b.nneg = __shfl_down_sync(0xffffffffu, a.nneg, o);
    diag_merge(a, b);
}

// block reduction in a fixed order: lanes by shuffle tree, warps in order
__device__ void diag_block(DiagAcc &a, double *out)
{
    __shared__ DiagAcc part[kDiagThreads / 32];
    for (int o = 16; o > 0; o >>= 1) diag_shfl(a, o);
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) part[w] = a;
    __syncthreads();
    if (threadIdx.x == 0) {
        DiagAcc r = part[0];
        for (int i = 1; i < (int)(blockDim.x >> 5); ++i) diag_merge(r, part[i]);
#pragma unroll
        for (int i = 0; i < 5; ++i) out[i] = r.s[i];
        out[5] = r.divb;
        out[6] = r.pmin;
        out[7] = r.nneg;
    }
}

__device__ __forceinline__ void diag_init(DiagAcc &a)
{
#pragma unroll
    for (int i = 0; i < 5; ++i) a.s[i] = 0.0;
    a.divb = 0.0;
    a.pmin = 1.0e300;
    a.nneg = 0.0;
}

__global__ void __launch_bounds__(kDiagThreads)
diag_kernel(const float *__restrict__ u, const float *__restrict__ b, int nx, int ny, int nz,
            double *__restrict__ part)
{
    DiagAcc a;
    diag_init(a);
    const long long ncell = (long long)nx * ny * nz;
    const double gm1 = (double)kGamma - 1.0;
    for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell;
         c += (long long)gridDim.x * blockDim.x) {
        const long long pen = c / nx;
        const int i = (int)(c - pen * nx);
        const int j = (int)(pen % ny), k = (int)(pen / ny);
        const long long cx = c + ((i + 1 == nx) ? -(long long)(nx - 1) : 1);
        const long long cy = c + ((j + 1 == ny) ? -(long long)(ny - 1) * nx : nx);
        const long long cz = c + ((k + 1 == nz) ? -(long long)(nz - 1) * nx * ny : (long long)nx * ny);
        double uu[5];
#pragma unroll
        for (int q = 0; q < 5; ++q) {
            uu[q] = (double)__ldg(u + c * 5 + q);
            a.s[q] += uu[q];
        }
        const double b0 = __ldg(b + c * 3 + 0), b1 = __ldg(b + c * 3 + 1), b2 = __ldg(b + c * 3 + 2);
        const double bx1 = __ldg(b + cx * 3 + 0), by1 = __ldg(b + cy * 3 + 1), bz1 = __ldg(b + cz * 3 + 2);
        a.divb = fmax(a.divb, fabs((bx1 - b0) + (by1 - b1) + (bz1 - b2)));
        const double cbx = 0.5 * (b0 + bx1), cby = 0.5 * (b1 + by1), cbz = 0.5 * (b2 + bz1);
        const double q = (uu[1] * uu[1] + uu[2] * uu[2] + uu[3] * uu[3]) / uu[0];
        const double p = gm1 * (uu[4] - 0.5 * q - 0.5 * (cbx * cbx + cby * cby + cbz * cbz));
        a.pmin = fmin(a.pmin, p);
        if (!(p > 0.0)) a.nneg += 1.0;
    }
    diag_block(a, part + (size_t)blockIdx.x * 8);
}

__global__ void __launch_bounds__(kDiagThreads)
diag_finish_kernel(const double *__restrict__ part, int nblocks, double *__restrict__ out)
{
    // one block: thread t folds partials t, t + 256, ... in order, then the block tree
    DiagAcc a;
    diag_init(a);
    for (int i = threadIdx.x; i < nblocks; i += blockDim.x) {
        DiagAcc b;
        const double *p = part + (size_t)i * 8;
#pragma unroll
        for (int q = 0; q < 5; ++q) b.s[q] = p[q];
        b.divb = p[5];
        b.pmin = p[6];
        b.nneg = p[7];
        diag_merge(a, b);
    }
    diag_block(a, out);
}

static int diag_blocks(long long ncell)
{
    long long g = (ncell + kDiagThreads - 1) / kDiagThreads;
    if (g > kDiagBlocksMax) g = kDiagBlocksMax;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace mhd

using namespace mhd;

extern "C" {

size_t mhdgpu_diagnostics_scratch_bytes(int nx, int ny, int nz)
{
    if (nx < 1 || ny < 1 || nz < 1) return 0;
    return sizeof(double) * 8 * (size_t)diag_blocks((long long)nx * ny * nz);
}

int mhdgpu_diagnostics(const float *u, const float *b, int nx, int ny, int nz, double *d_out,
                       void *d_scratch, mhdgpu_stream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || (long long)nx * ny * nz > (1LL << 31)) {
        set_last_error("mhdgpu_diagnostics: bad box");
        return MHD_ERR_ARG;
    }
    if (!u || !b || !d_out || !d_scratch) {
        set_last_error("mhdgpu_diagnostics: null pointer");
        return MHD_ERR_ARG;
    }
    cudaStream_t s = (cudaStream_t)stream;
    const int g = diag_blocks((long long)nx * ny * nz);
    double *part = (double *)d_scratch;
    diag_kernel<<<g, kDiagThreads, 0, s>>>(u, b, nx, ny, nz, part);
    diag_finish_kernel<<<1, kDiagThreads, 0, s>>>(part, g, d_out);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_last_error(cudaGetErrorString(e));
        return MHD_ERR_CUDA;
    }
    return MHD_OK;
}

}  // extern "C"
