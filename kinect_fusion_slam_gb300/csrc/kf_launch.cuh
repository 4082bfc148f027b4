// Kernel launches with programmatic dependent launch: the next kernel in the stream is
// scheduled while this one drains, and waits (griddepcontrol.wait) for it to finish
// before touching anything it produced.  Hides the launch gap between the frame's
// dependent kernels, inside and outside CUDA graphs.
#pragma once

#include <cuda_runtime.h>

namespace kf {

// first statement of every kernel launched with launch_pdl
__device__ __forceinline__ void wait_for_producer() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <class... KArgs, class... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, Args&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

}  // namespace kf
