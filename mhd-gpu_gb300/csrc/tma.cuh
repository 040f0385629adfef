// tma.cuh - the Tensor Memory Accelerator (TMA) plumbing of the row-staged
// sweeps: mbarrier completion, 3-D tiled bulk tensor copies between global and
// shared memory, and the host-side tensor-map encoding.
//
// A sweep along y or z of a box stored x-major reads pencils that run across
// memory.  A CTA owns P neighbouring pencils at one plane k; row i of its tile
// is P consecutive cells of the frame's j axis, one contiguous run of 5P
// floats of u (3P of b).  One tensor copy moves the whole tile (N rows of 5P
// floats) into shared memory as [i][5P], issued by one thread and completed on
// an mbarrier; the write-back is one tensor store of the same box.  The
// tensor maps describe u and b as 3-D arrays (j and the components fused into
// the contiguous dimension, then the frame's i and k axes with their strides),
// so the y and z frames differ only in their strides.
//
// Every wait here is bounded: a wait that gives up reports it to the caller,
// which flags the box's health word and waits, bounded again, for its copies
// in flight before it moves on.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace mhd {

// ---------------------------------------------------------------- device side

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// makes the initialised barrier visible to the async proxy (the TMA unit)
__device__ __forceinline__ void mbar_init_fence()
{
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

// one probe of the barrier's phase `parity`; true once that phase completed
__device__ __forceinline__ bool mbar_test(uint64_t *bar, unsigned parity)
{
    unsigned done;
    asm volatile(
        "{\n"
        ".reg .pred p;\n"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        "selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(done)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// Waits for phase `parity` of the barrier, at most ~2^22 probes (each probe
// itself suspends for a hardware-bounded time, and a sleep separates them):
// returns false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity)
{
    if (mbar_test(bar, parity)) return true;
    for (int it = 0; it < (1 << 22); ++it) {
        __nanosleep(64);
        if (mbar_test(bar, parity)) return true;
    }
    return false;
}

// generic-proxy accesses of shared memory before this fence are ordered
// before later async-proxy (TMA) accesses of it, and conversely
__device__ __forceinline__ void fence_proxy_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// 3-D tiled load of the box at (x, y, z) into shared memory, completing its
// bytes on the barrier (the caller arms the barrier with the total)
__device__ __forceinline__ void tma_load_3d(void *smem_dst, const CUtensorMap *map, int x, int y, int z,
                                            uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];\n" ::"r"(smem_u32(smem_dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// 3-D tiled store of a shared-memory box to (x, y, z); elements outside the
// tensor are not written.  Completion through the bulk async-group.
__device__ __forceinline__ void tma_store_3d(const CUtensorMap *map, int x, int y, int z, const void *smem_src)
{
    asm volatile(
        "cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];\n" ::"l"(
            reinterpret_cast<uint64_t>(map)),
        "r"(x), "r"(y), "r"(z), "r"(smem_u32(smem_src))
        : "memory");
}

__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;\n" ::: "memory"); }

// the stores committed so far have read their shared-memory source
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;\n" ::: "memory"); }

// the stores committed so far are complete (their global writes performed)
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;\n" ::: "memory"); }

// ---------------------------------------------------------------- host side

// The four maps of one row-staged frame of one box: u (box 5P x N x 1), b
// with the j+1 column (3P+4 floats wide), b of the k+1 plane (3P wide) and b
// of column 0 (4 wide, the periodic j+1 of the last column).
struct RowMaps {
    CUtensorMap u, b, bk, bw;
};

// Whether a frame of a box can be row-staged through TMA with P pencils per
// tile: every global stride a multiple of 16 bytes, P a multiple of 4, the
// pencil length and the tile width within the 256-element box limit, and the
// arrays 16-byte aligned.
bool tma_rows_ok(const float *u, const float *b, int n, int ny, int nz, long long si, long long sk, int P);

// Encodes the four maps (returns false when the driver refuses one).
bool tma_rows_encode(RowMaps *m, const float *u, const float *b, int n, int ny, int nz, long long si,
                     long long sk, int P);

}  // namespace mhd
