// profiler.cuh - hooks the C-ABI entries use to record CUDA events around
// their launches when a profiler is attached to the calling thread.
#pragma once

#include <cuda_runtime.h>

namespace mhd {

// returns a slot (or -1 when no profiler is attached or it is full)
int prof_begin(int kclass, int launches, cudaStream_t s);
void prof_end(int slot, cudaStream_t s);

struct ProfScope {
    int slot;
    cudaStream_t s;
    ProfScope(int kclass, int launches, cudaStream_t st) : slot(prof_begin(kclass, launches, st)), s(st) {}
    ~ProfScope() { prof_end(slot, s); }
};

}  // namespace mhd
