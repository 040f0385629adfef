// profiler.cu - per-kernel-class CUDA-event timing for the C ABI.
//
// A profiler attached to the calling thread makes every C-ABI entry that
// launches kernels record a start and an end event on the caller's stream
// around its launches, so per-launch device durations can be read inside a
// real run (stream order is unchanged; no synchronisation is added).  The
// reference only timed whole steps with events (Cuda/cuda_main.cu:68-77,
// 122-128) and OpenCL marker kernels (OpenCL/backup_OpenCL_mhd/mhd_run.cpp:200-280).
#include <cuda_runtime.h>
#include <stdio.h>

#include <nvtx3/nvToolsExt.h>

#include <vector>

#include "mhdgpu.h"
#include "profiler.cuh"

struct mhdgpu_profiler {
    struct Rec { cudaEvent_t a, b; int kclass; int launches; };
    std::vector<Rec> recs;
    int used = 0;
    int dropped = 0;
};

namespace mhd {

static thread_local mhdgpu_profiler *g_prof = nullptr;

int prof_begin(int kclass, int launches, cudaStream_t s)
{
    mhdgpu_profiler *p = g_prof;
    if (!p) return -1;
    if (p->used >= (int)p->recs.size()) { p->dropped++; return -1; }
    const int slot = p->used++;
    p->recs[slot].kclass = kclass;
    p->recs[slot].launches = launches;
    cudaEventRecord(p->recs[slot].a, s);
    return slot;
}

void prof_end(int slot, cudaStream_t s)
{
    mhdgpu_profiler *p = g_prof;
    if (!p || slot < 0) return;
    cudaEventRecord(p->recs[slot].b, s);
}

void nvtx_push(int kclass)
{
    static const char *const names[] = {"mhdgpu fluidx", "mhdgpu advectbyzx", "mhdgpu transpose",
                                        "mhdgpu cfl", "mhdgpu batch sweep"};
    nvtxRangePushA(kclass >= 0 && kclass < 5 ? names[kclass] : "mhdgpu");
}

void nvtx_pop() { nvtxRangePop(); }

}  // namespace mhd

extern "C" {

int mhdgpu_profiler_create(mhdgpu_profiler **out, int max_records)
{
    if (!out || max_records < 1) return MHD_ERR_ARG;
    mhdgpu_profiler *p = new mhdgpu_profiler;
    p->recs.resize(max_records);
    for (auto &r : p->recs) {
        if (cudaEventCreate(&r.a) != cudaSuccess || cudaEventCreate(&r.b) != cudaSuccess) {
            delete p;
            return MHD_ERR_CUDA;
        }
        r.kclass = -1;
        r.launches = 0;
    }
    *out = p;
    return MHD_OK;
}

int mhdgpu_profiler_destroy(mhdgpu_profiler *p)
{
    if (!p) return MHD_ERR_ARG;
    if (mhd::g_prof == p) mhd::g_prof = nullptr;
    for (auto &r : p->recs) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    delete p;
    return MHD_OK;
}

int mhdgpu_profiler_attach(mhdgpu_profiler *p)
{
    mhd::g_prof = p;
    return MHD_OK;
}

int mhdgpu_profiler_reset(mhdgpu_profiler *p)
{
    if (!p) return MHD_ERR_ARG;
    p->used = 0;
    p->dropped = 0;
    return MHD_OK;
}

int mhdgpu_profiler_summary(mhdgpu_profiler *p, int kclass, int *records, int *launches,
                            double *total_ms)
{
    if (!p || kclass < 0 || kclass >= MHD_KCLASS_COUNT) return MHD_ERR_ARG;
    int nrec = 0, nl = 0;
    double ms = 0.0;
    for (int i = 0; i < p->used; ++i) {
        auto &r = p->recs[i];
        if (r.kclass != kclass) continue;
        if (cudaEventSynchronize(r.b) != cudaSuccess) return MHD_ERR_CUDA;
        float t = 0.0f;
        if (cudaEventElapsedTime(&t, r.a, r.b) != cudaSuccess) return MHD_ERR_CUDA;
        ms += t;
        nrec++;
        nl += r.launches;
    }
    if (records) *records = nrec;
    if (launches) *launches = nl;
    if (total_ms) *total_ms = ms;
    return p->dropped ? MHD_ERR_ARG : MHD_OK;
}

}  // extern "C"
