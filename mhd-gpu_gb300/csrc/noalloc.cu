// noalloc.cu - mhdgpu_advectbyzx_noalloc: the advectbyzx step for callers that
// cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is not available or not
// allowed at the point of the call -- a plugin invoked from inside another
// runtime's memory pool, a real-time loop that must not take the allocator's
// locks or risk an out-of-memory error mid-run, or a host that hands this
// library nothing but its own input and output buffers.  mhdgpu_advectbyzx
// needs two floats of scratch per cell from its caller; this variant keeps
// that scratch in a fixed array in the library's own device memory instead.
//
// The array is a file-scope __device__ object of MHD_NOALLOC_MAX_CELLS * 2
// floats (16 MiB).  Every GPU that loads this library holds it until the
// process exits.  Its name is only a host-side stand-in in host code, so the
// device address is looked up once per device with cudaGetSymbolAddress, with
// that device current, on the first call made while it is the current device;
// make that first call before any stream capture.  mhdgpu_release_host_cache
// forgets the looked-up addresses (a device reset unloads the module and the
// array may come back elsewhere), so the next call looks them up again.
// Every call shares the one
// array: calls that overlap on the GPU (different streams, or threads using
// the same device) race on it and must be serialised by the caller.  The
// flux kernel writes every scratch entry it covers before the gather kernel
// reads any, so no part of the array has to start at zero and nothing is
// cleared between calls.
#include <cuda_runtime.h>
#include <stdio.h>

#include <mutex>

#include "kernels.cuh"
#include "profiler.cuh"

namespace {

static __device__ __align__(256) float g_advect_scratch[2 * (size_t)MHD_NOALLOC_MAX_CELLS];

constexpr int kMaxDevices = 64;
float *g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_setup_mutex;

int noalloc_fail(int status, const char *msg)
{
    mhd::set_last_error(msg);
    return status;
}

int noalloc_cuda_fail(const char *where, cudaError_t e)
{
    char buf[256];
    snprintf(buf, sizeof buf, "mhdgpu_advectbyzx_noalloc: %s: %s", where, cudaGetErrorString(e));
    mhd::set_last_error(buf);
    return MHD_ERR_CUDA;
}

// Device address of the scratch array on the current device (looked up once).
int scratch_on_current_device(float **out)
{
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return noalloc_cuda_fail("cudaGetDevice", e);
    if (dev < 0 || dev >= kMaxDevices)
        return noalloc_fail(MHD_ERR_ARG, "mhdgpu_advectbyzx_noalloc: device ordinal above 63");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_advect_scratch);
        if (e != cudaSuccess) return noalloc_cuda_fail("cudaGetSymbolAddress", e);
        if (!p) return noalloc_fail(MHD_ERR_CUDA, "mhdgpu_advectbyzx_noalloc: scratch address is null");
        g_scratch_ptr[dev] = static_cast<float *>(p);
    }
    *out = g_scratch_ptr[dev];
    return MHD_OK;
}

}  // namespace

// Called by mhdgpu_release_host_cache: after a device reset the array's old
// address is no longer valid, so every device looks it up again.
void mhd::noalloc_forget_devices()
{
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    for (int d = 0; d < kMaxDevices; ++d) g_scratch_ptr[d] = nullptr;
}

extern "C" {

int mhdgpu_advectbyzx_noalloc(float *b, const float *u, int nx, int ny, int nz, const float *d_dt,
                              mhdgpu_stream_t stream)
{
    if (nx < 1 || ny < 1 || nz < 1 || nx > MHD_MAX_PENCIL)
        return noalloc_fail(MHD_ERR_ARG, "mhdgpu_advectbyzx_noalloc: bad box (each axis >= 1, nx <= 1024)");
    const long long ncell = (long long)nx * ny * nz;
    if (ncell > (long long)MHD_NOALLOC_MAX_CELLS)
        return noalloc_fail(MHD_ERR_ARG,
                            "mhdgpu_advectbyzx_noalloc: box has more than MHD_NOALLOC_MAX_CELLS "
                            "(2097152) cells; use mhdgpu_advectbyzx with caller scratch");
    if (!b || !u || !d_dt) return noalloc_fail(MHD_ERR_ARG, "mhdgpu_advectbyzx_noalloc: null pointer");
    float *scr = nullptr;
    int st = scratch_on_current_device(&scr);
    if (st != MHD_OK) return st;
    mhd::AdvectArgs a = mhd::make_advect_args(b, u, d_dt, scr, scr + ncell, mhd::make_frame(nx, ny, nz));
    mhd::ProfScope ps(MHD_KCLASS_ADVECT, 2, (cudaStream_t)stream);
    cudaError_t e = mhd::launch_advect(a, mhd::pencil_cfg(MHD_KCLASS_ADVECT, nx), mhd::math_mode(), (cudaStream_t)stream);
    if (e != cudaSuccess) return noalloc_cuda_fail("launch", e);
    return MHD_OK;
}

}  // extern "C"
