// Programmatic dependent launch (PTX griddepcontrol, sm_90 and later).
//
// A kernel launched with cudaLaunchAttributeProgrammaticStreamSerialization may start before the
// kernel ahead of it in the stream has finished: once every block of that kernel has executed
// griddepcontrol.launch_dependents (or exited), the dependent grid's blocks are scheduled into the
// SM slots the earlier grid leaves.  A dependent thread must execute griddepcontrol.wait before it
// touches memory the earlier grid writes or reads: the wait returns once the earlier grid has
// completed and its memory operations are visible.  Without a prerequisite grid (a launch without
// the attribute, or after a copy) the wait returns at once, and launch_dependents is a no-op when
// the next launch does not carry the attribute.
//
// No block ever waits on a block of its own grid, and a dependent grid is launched only after
// every block of the earlier grid has started, so the earlier grid always runs to completion.
#pragma once

#include <cuda_runtime.h>

namespace lbm {

__device__ __forceinline__ void allow_dependent_launch() {
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

__device__ __forceinline__ void wait_prerequisite_grids() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Launch `kernel` on `stream`, as a programmatic dependent of the kernel ahead of it when
// `dependent` is true.
template <class... Params, class... Args>
cudaError_t launch_maybe_dependent(bool dependent, void (*kernel)(Params...), dim3 grid, dim3 block, size_t smem,
                                   cudaStream_t stream, Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = dependent ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<Args &&>(args)...);
}

}  // namespace lbm
