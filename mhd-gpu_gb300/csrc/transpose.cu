// transpose.cu - the axis permutations transpose12 and transpose13 with their
// component permutations, for sm_103a.  Pure copies: bit-exact.
//
// transpose12: Heterogeneous_MHD/C/transpose12.c:7-47 (OpenMP/mhd.f90:410-430)
//   dst(ii, j, i, k) = src(perm12[ii], i, j, k), u perm (1,3,2,4,5), b perm (2,1,3)
// transpose13: Heterogeneous_MHD/C/transpose13.c:9-62 (OpenMP/mhd.f90:433-474)
//   dst(ii, k, j, i) = src(perm13[ii], i, j, k), u perm (1,4,3,2,5), b perm (3,2,1)
// The reference accepts transpose13 only for nx == nz (or the Fortran
// special cases nz == 1 / nx == 1, which reduce to the same formula); this
// kernel applies the formula to every shape.
//
// Both are one kernel: a 32x32-cell tile of the (a, b) plane, a = the source's
// fast axis i, b = the axis that becomes the destination's fast axis, and an
// outer axis o.  Rows of 32 cells (160 floats of u, 96 of b) are read and
// written with consecutive threads on consecutive addresses; the tile rows in
// shared memory are padded to a stride of 5 (u) or 3 (b) banks mod 32 so the
// transposed read is conflict-free.
#include "kernels.cuh"

namespace mhd {

struct TransposeArgs {
    float *du, *db;
    const float *su, *sb;
    int A, B, O;                 // extents of a, b, o
    long long sb_in, so_in;      // source cell strides of b and o (a has stride 1)
    long long sa_out, so_out;    // destination cell strides of a and o (b has stride 1)
    unsigned pu, pb;             // destination component ii <- source component
                                 // (p >> 4*ii) & 15 (packed so no local array)
};

constexpr int kTile = 32;
constexpr int kRowU = kTile * 5 + 5;   // 165 = 5 mod 32
constexpr int kRowB = kTile * 3 + 3;   // 99  = 3 mod 32

__global__ void __launch_bounds__(256)
transpose_kernel(TransposeArgs t)
{
    __shared__ float tu[kTile * kRowU];
    __shared__ float tb[kTile * kRowB];
    const int a0 = blockIdx.x * kTile;
    const int b0 = blockIdx.y * kTile;
    const long long o = blockIdx.z;
    const int na = min(kTile, t.A - a0);
    const int nb = min(kTile, t.B - b0);

    // load: tile row r = source row b0+r, 32 cells along a
    for (int e = threadIdx.x; e < kTile * kTile * 5; e += blockDim.x) {
        const int r = e / (kTile * 5), col = e - r * (kTile * 5);
        if (r < nb && col < na * 5) {
            const long long cell = (long long)a0 + (long long)(b0 + r) * t.sb_in + o * t.so_in;
            tu[r * kRowU + col] = t.su[cell * 5 + col];
        }
    }
    for (int e = threadIdx.x; e < kTile * kTile * 3; e += blockDim.x) {
        const int r = e / (kTile * 3), col = e - r * (kTile * 3);
        if (r < nb && col < na * 3) {
            const long long cell = (long long)a0 + (long long)(b0 + r) * t.sb_in + o * t.so_in;
            tb[r * kRowB + col] = t.sb[cell * 3 + col];
        }
    }
    __syncthreads();
    // store: destination row s = source column a0+s, 32 cells along b
    for (int e = threadIdx.x; e < kTile * kTile * 5; e += blockDim.x) {
        const int s = e / (kTile * 5), col = e - s * (kTile * 5);
        const int bb = col / 5, cc = col - bb * 5;
        if (s < na && bb < nb) {
            const long long cell = (long long)b0 + (long long)(a0 + s) * t.sa_out + o * t.so_out;
            t.du[cell * 5 + col] = tu[bb * kRowU + s * 5 + ((t.pu >> (4 * cc)) & 15u)];
        }
    }
    for (int e = threadIdx.x; e < kTile * kTile * 3; e += blockDim.x) {
        const int s = e / (kTile * 3), col = e - s * (kTile * 3);
        const int bb = col / 3, cc = col - bb * 3;
        if (s < na && bb < nb) {
            const long long cell = (long long)b0 + (long long)(a0 + s) * t.sa_out + o * t.so_out;
            t.db[cell * 3 + col] = tb[bb * kRowB + s * 3 + ((t.pb >> (4 * cc)) & 15u)];
        }
    }
}

cudaError_t launch_transpose(float *du, float *db, const float *su, const float *sb,
                             int nx, int ny, int nz, int which, cudaStream_t s)
{
    TransposeArgs t;
    t.du = du; t.db = db; t.su = su; t.sb = sb;
    if (which == 12) {
        // a = i (nx), b = j (ny), o = k (nz); destination dims (ny, nx, nz)
        t.A = nx; t.B = ny; t.O = nz;
        t.sb_in = nx; t.so_in = (long long)nx * ny;
        t.sa_out = ny; t.so_out = (long long)nx * ny;
        t.pu = 0x43120u;   // (0, 2, 1, 3, 4)
        t.pb = 0x201u;     // (1, 0, 2)
    } else {
        // a = i (nx), b = k (nz), o = j (ny); destination dims (nz, ny, nx)
        t.A = nx; t.B = nz; t.O = ny;
        t.sb_in = (long long)nx * ny; t.so_in = nx;
        t.sa_out = (long long)ny * nz; t.so_out = nz;
        t.pu = 0x41230u;   // (0, 3, 2, 1, 4)
        t.pb = 0x012u;     // (2, 1, 0)
    }
    if (t.O > 65535) return cudaErrorInvalidConfiguration;
    dim3 grid((t.A + kTile - 1) / kTile, (t.B + kTile - 1) / kTile, t.O);
    transpose_kernel<<<grid, 256, 0, s>>>(t);
    return cudaGetLastError();
}

}  // namespace mhd
