// tma.cu - host side of the TMA row staging (tma.cuh): tensor-map encoding
// through the driver entry point (the library links only the CUDA runtime).
#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <mutex>

#include "tma.cuh"

namespace mhd {

namespace {

typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *,
                                  CUtensorMapInterleave, CUtensorMapSwizzle, CUtensorMapL2promotion,
                                  CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn()
{
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    return fn;
}

// one 3-D float map: dims (w, n, nz) with w contiguous, strides (bytes) of the
// second and third dimensions, box (bw, n, 1); out-of-bounds reads fill zeros
bool encode3(CUtensorMap *m, const float *base, unsigned long long w, int n, int nz, unsigned long long s1,
             unsigned long long s2, unsigned bw)
{
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    const cuuint64_t dims[3] = {w, (cuuint64_t)n, (cuuint64_t)nz};
    const cuuint64_t strides[2] = {s1, s2};
    const cuuint32_t box[3] = {bw, (cuuint32_t)n, 1};
    const cuuint32_t estr[3] = {1, 1, 1};
    return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float *>(base), dims, strides, box, estr,
              CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
              CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

}  // namespace

bool tma_rows_ok(const float *u, const float *b, int n, int ny, int nz, long long si, long long sk, int P)
{
    if (!encode_fn()) return false;
    if (P < 4 || P % 4 != 0 || 5 * P > 256 || 3 * P + 4 > 256) return false;
    if (n < 1 || n > 256 || ny < 1 || nz < 1) return false;
    if (((reinterpret_cast<uintptr_t>(u) | reinterpret_cast<uintptr_t>(b)) & 15u) != 0) return false;
    // strides in bytes: u rows 20 si, planes 20 sk; b rows 12 si, planes 12 sk
    if ((si % 4) != 0 || (sk % 4) != 0) return false;
    const long long lim = 1LL << 40;
    return 20 * si < lim && 20 * sk < lim;
}

bool tma_rows_encode(RowMaps *m, const float *u, const float *b, int n, int ny, int nz, long long si,
                     long long sk, int P)
{
    if (!tma_rows_ok(u, b, n, ny, nz, si, sk, P)) return false;
    const unsigned long long wu = 5ull * ny, wb = 3ull * ny;
    return encode3(&m->u, u, wu, n, nz, 20ull * si, 20ull * sk, 5u * P) &&
           encode3(&m->b, b, wb, n, nz, 12ull * si, 12ull * sk, 3u * P + 4u) &&
           encode3(&m->bk, b, wb, n, nz, 12ull * si, 12ull * sk, 3u * P) &&
           encode3(&m->bw, b, wb, n, nz, 12ull * si, 12ull * sk, 4u);
}

}  // namespace mhd
