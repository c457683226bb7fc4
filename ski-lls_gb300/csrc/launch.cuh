// launch.cuh -- kernel launches with programmatic dependent launch (PDL).
//
// A kernel launched through launch_k may start (be scheduled, run its
// prologue) while the kernel before it on the same stream drains; it waits in
// pdl_wait() -- griddepcontrol.wait, the first statement of every kernel
// launched this way -- until that kernel has completed and its writes are
// visible.  On a chain of dependent small kernels this hides the ~2.7 us the
// GPU otherwise spends between one kernel's end and the next one's start
// (measured on GB300: 4.1 -> 1.4 us per launch of an empty kernel).  Without
// a programmatic predecessor pdl_wait() returns at once.  SKILLS_PDL=0 turns
// the attribute off (for comparison).
#pragma once
#include <cstdlib>
#include <utility>

#include <cuda_runtime.h>

#include "skl_internal.hpp"

namespace skl {

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

inline bool pdl_enabled()
{
    static const bool v = [] {
        const char* e = getenv("SKILLS_PDL");
        return !(e && e[0] == '0');
    }();
    return v;
}

template <typename... KArgs, typename... Args>
inline void launch_k(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
                     Args&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = pdl_enabled() ? 1 : 0;
    SKL_CUDA(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...));
}

}  // namespace skl
