// mhd_debug.cuh - index checks of the debug build.
//
// Built with -DMHD_DEBUG (build.py --debug: lib/libmhdgpu_debug.so), every
// shared-memory, global and halo index of the kernels is checked where it is
// formed: an index outside its array records the site and is skipped (a load
// reads 0, a store or copy does not happen), so a bad index never faults the
// GPU and the host reads the first one back with mhdgpu_debug_faults.  In the
// release build the checks are the constant `true` and vanish.
//
//   MHD_IN(i, n)        0 <= i < n (an index into an array of n elements)
//   MHD_SM(p, bytes)    [p, p+bytes) lies in the launch's dynamic shared memory
//   MHD_GM(p, lo, n)    p lies in the global array of n floats at lo
//
// A site is the file (MHD_DBG_FILE, set by each checked file after its
// includes) and the line.
#pragma once

#include <stdint.h>

namespace mhd {

enum { kDbgIndex = 1, kDbgShared = 2, kDbgGlobal = 3 };

#if defined(MHD_DEBUG)

// the first fault and the number of faults since the last read (debug.cu)
extern __device__ unsigned g_dbg_count;
extern __device__ unsigned g_dbg_site;   // kind << 28 | file << 20 | line
extern __device__ long long g_dbg_index, g_dbg_extent;

__device__ __noinline__ bool debug_fault(unsigned kind, unsigned file, unsigned line, long long index,
                                         long long extent);

__device__ __forceinline__ bool debug_in(long long i, long long n, unsigned file, unsigned line)
{
    return (i >= 0 && i < n) ? true : debug_fault(kDbgIndex, file, line, i, n);
}

__device__ __forceinline__ bool debug_smem(const void *p, unsigned bytes, unsigned file, unsigned line)
{
    extern __shared__ float mhd_dbg_dynamic_smem[];   // the start of the dynamic area
    unsigned dyn;
    asm("mov.u32 %0, %%dynamic_smem_size;" : "=r"(dyn));
    const long long lo = (long long)__cvta_generic_to_shared(mhd_dbg_dynamic_smem);
    const long long off = (long long)__cvta_generic_to_shared(p) - lo;
    return (off >= 0 && off + bytes <= (long long)dyn) ? true : debug_fault(kDbgShared, file, line, off, dyn);
}

__device__ __forceinline__ bool debug_gmem(const void *p, const float *lo, long long n, unsigned file, unsigned line)
{
    const long long off = reinterpret_cast<const float *>(p) - lo;
    return (off >= 0 && off < n) ? true : debug_fault(kDbgGlobal, file, line, off, n);
}

#define MHD_IN(i, n) ::mhd::debug_in((long long)(i), (long long)(n), MHD_DBG_FILE, __LINE__)
#define MHD_SM(p, bytes) ::mhd::debug_smem((p), (bytes), MHD_DBG_FILE, __LINE__)
#define MHD_GM(p, lo, n) ::mhd::debug_gmem((p), (lo), (long long)(n), MHD_DBG_FILE, __LINE__)

#else

#define MHD_IN(i, n) true
#define MHD_SM(p, bytes) true
#define MHD_GM(p, lo, n) true

#endif

}  // namespace mhd
