// profiler.cuh - hooks the C-ABI entries use to record CUDA events around
// their launches when a profiler is attached to the calling thread.
#pragma once

#include <cuda_runtime.h>

namespace mhd {

// returns a slot (or -1 when no profiler is attached or it is full)
int prof_begin(int kclass, int launches, cudaStream_t s);
void prof_end(int slot, cudaStream_t s);
// an NVTX range named after the kernel class, for timeline tools (nsys,
// ncu --nvtx); without such a tool attached the calls do nothing
void nvtx_push(int kclass);
void nvtx_pop();

// Around the launches of one C-ABI entry: the CUDA-event record of an
// attached profiler and an NVTX range.
struct ProfScope {
    int slot;
    cudaStream_t s;
    ProfScope(int kclass, int launches, cudaStream_t st) : slot(prof_begin(kclass, launches, st)), s(st)
    {
        nvtx_push(kclass);
    }
    ~ProfScope()
    {
        prof_end(slot, s);
        nvtx_pop();
    }
};

}  // namespace mhd
