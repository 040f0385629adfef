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
// transposed read is conflict-free.  A full tile whose rows start on 16-byte
// boundaries (the strides along b and o multiples of 4 cells, 16-byte aligned
// arrays) moves 16-byte vectors, all of a thread's loads issued before its
// shared-memory stores; other tiles move single floats.
#include "kernels.cuh"

#undef MHD_DBG_FILE
#define MHD_DBG_FILE 6

namespace mhd {

struct TransposeArgs {
    float *du, *db;
    const float *su, *sb;
    int A, B, O;                 // extents of a, b, o
    long long sb_in, so_in;      // source cell strides of b and o (a has stride 1)
    long long sa_out, so_out;    // destination cell strides of a and o (b has stride 1)
    unsigned pu, pb;             // destination component ii <- source component
                                 // (p >> 4*ii) & 15 (packed so no local array)
    int vec;                     // full tiles may move 16-byte vectors
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
    // cells of the box (the debug build's extent for global indices)
#define MHD_TNC ((long long)t.A * t.B * t.O)

    if (t.vec && na == kTile && nb == kTile) {
        // u: 32 rows x 40 vectors, b: 32 rows x 24 vectors; 256 threads
        constexpr int kVu = kTile * kTile * 5 / 4 / 256, kVb = kTile * kTile * 3 / 4 / 256;
        float4 lu[kVu], lb[kVb];
#pragma unroll
        for (int k = 0; k < kVu; ++k) {
            const int e = threadIdx.x + 256 * k, r = e / 40, c = e - r * 40;
            const long long cell = (long long)a0 + (long long)(b0 + r) * t.sb_in + o * t.so_in;
            lu[k] = MHD_GM(t.su + cell * 5 + 4 * c + 3, t.su, 5 * MHD_TNC)
                        ? __ldg(reinterpret_cast<const float4 *>(t.su + cell * 5) + c)
                        : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
#pragma unroll
        for (int k = 0; k < kVb; ++k) {
            const int e = threadIdx.x + 256 * k, r = e / 24, c = e - r * 24;
            const long long cell = (long long)a0 + (long long)(b0 + r) * t.sb_in + o * t.so_in;
            lb[k] = MHD_GM(t.sb + cell * 3 + 4 * c + 3, t.sb, 3 * MHD_TNC)
                        ? __ldg(reinterpret_cast<const float4 *>(t.sb + cell * 3) + c)
                        : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        }
#pragma unroll
        for (int k = 0; k < kVu; ++k) {
            const int e = threadIdx.x + 256 * k, r = e / 40, c = e - r * 40;
            float *d = tu + r * kRowU + 4 * c;
            if (!MHD_IN(r * kRowU + 4 * c + 3, kTile * kRowU)) continue;
            d[0] = lu[k].x; d[1] = lu[k].y; d[2] = lu[k].z; d[3] = lu[k].w;
        }
#pragma unroll
        for (int k = 0; k < kVb; ++k) {
            const int e = threadIdx.x + 256 * k, r = e / 24, c = e - r * 24;
            float *d = tb + r * kRowB + 4 * c;
            if (!MHD_IN(r * kRowB + 4 * c + 3, kTile * kRowB)) continue;
            d[0] = lb[k].x; d[1] = lb[k].y; d[2] = lb[k].z; d[3] = lb[k].w;
        }
        __syncthreads();
        // destination row s: floats 4c .. 4c+3 of the row are (cell, component)
        // pairs (col / 5, col % 5) of u, (col / 3, col % 3) of b
#pragma unroll
        for (int k = 0; k < kVu; ++k) {
            const int e = threadIdx.x + 256 * k, s = e / 40, c = e - s * 40;
            float v[4];
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const int col = 4 * c + m, bb = col / 5, cc = col - bb * 5;
                const int x = bb * kRowU + s * 5 + ((t.pu >> (4 * cc)) & 15u);
                v[m] = MHD_IN(x, kTile * kRowU) ? tu[x] : 0.0f;
            }
            const long long cell = (long long)b0 + (long long)(a0 + s) * t.sa_out + o * t.so_out;
            if (MHD_GM(t.du + cell * 5 + 4 * c + 3, t.du, 5 * MHD_TNC))
                reinterpret_cast<float4 *>(t.du + cell * 5)[c] = make_float4(v[0], v[1], v[2], v[3]);
        }
#pragma unroll
        for (int k = 0; k < kVb; ++k) {
            const int e = threadIdx.x + 256 * k, s = e / 24, c = e - s * 24;
            float v[4];
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                const int col = 4 * c + m, bb = col / 3, cc = col - bb * 3;
                const int x = bb * kRowB + s * 3 + ((t.pb >> (4 * cc)) & 15u);
                v[m] = MHD_IN(x, kTile * kRowB) ? tb[x] : 0.0f;
            }
            const long long cell = (long long)b0 + (long long)(a0 + s) * t.sa_out + o * t.so_out;
            if (MHD_GM(t.db + cell * 3 + 4 * c + 3, t.db, 3 * MHD_TNC))
                reinterpret_cast<float4 *>(t.db + cell * 3)[c] = make_float4(v[0], v[1], v[2], v[3]);
        }
        return;
    }

    // load: tile row r = source row b0+r, 32 cells along a
    for (int e = threadIdx.x; e < kTile * kTile * 5; e += blockDim.x) {
        const int r = e / (kTile * 5), col = e - r * (kTile * 5);
        if (r < nb && col < na * 5) {
            const long long cell = (long long)a0 + (long long)(b0 + r) * t.sb_in + o * t.so_in;
            if (MHD_IN(r * kRowU + col, kTile * kRowU) && MHD_GM(t.su + cell * 5 + col, t.su, 5 * MHD_TNC))
                tu[r * kRowU + col] = t.su[cell * 5 + col];
        }
    }
    for (int e = threadIdx.x; e < kTile * kTile * 3; e += blockDim.x) {
        const int r = e / (kTile * 3), col = e - r * (kTile * 3);
        if (r < nb && col < na * 3) {
            const long long cell = (long long)a0 + (long long)(b0 + r) * t.sb_in + o * t.so_in;
            if (MHD_IN(r * kRowB + col, kTile * kRowB) && MHD_GM(t.sb + cell * 3 + col, t.sb, 3 * MHD_TNC))
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
            const int x = bb * kRowU + s * 5 + ((t.pu >> (4 * cc)) & 15u);
            if (MHD_IN(x, kTile * kRowU) && MHD_GM(t.du + cell * 5 + col, t.du, 5 * MHD_TNC))
                t.du[cell * 5 + col] = tu[x];
        }
    }
    for (int e = threadIdx.x; e < kTile * kTile * 3; e += blockDim.x) {
        const int s = e / (kTile * 3), col = e - s * (kTile * 3);
        const int bb = col / 3, cc = col - bb * 3;
        if (s < na && bb < nb) {
            const long long cell = (long long)b0 + (long long)(a0 + s) * t.sa_out + o * t.so_out;
            const int x = bb * kRowB + s * 3 + ((t.pb >> (4 * cc)) & 15u);
            if (MHD_IN(x, kTile * kRowB) && MHD_GM(t.db + cell * 3 + col, t.db, 3 * MHD_TNC))
                t.db[cell * 3 + col] = tb[x];
        }
    }
#undef MHD_TNC
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
    // 16-byte rows: a row starts at cell a0 + b*sb_in + o*so_in (a0 a multiple
    // of 32), i.e. at byte 20 cell (u) or 12 cell (b), aligned when the cell
    // index is a multiple of 4; likewise for the destination rows
    auto al16 = [](const void *p) { return ((unsigned long long)p & 15ull) == 0; };
    t.vec = t.sb_in % 4 == 0 && t.so_in % 4 == 0 && t.sa_out % 4 == 0 && t.so_out % 4 == 0 &&
            al16(du) && al16(db) && al16(su) && al16(sb);
    if (t.O > 65535) return cudaErrorInvalidConfiguration;
    dim3 grid((t.A + kTile - 1) / kTile, (t.B + kTile - 1) / kTile, t.O);
    transpose_kernel<<<grid, 256, 0, s>>>(t);
    return cudaGetLastError();
}

}  // namespace mhd
