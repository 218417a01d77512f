// pdl.cuh -- programmatic dependent launch for the element-wise and reduction
// kernels, so that consecutive kernels of a stream overlap launch and tail.
//
// A kernel launched by launch_pdl may be scheduled before the previous kernel
// of its stream has finished.  pdl_enter() at the top of the kernel waits for
// that kernel to complete (its writes visible) before anything is read, then
// allows the next kernel to be scheduled.  The next grid is scheduled only
// when every CTA of this one has passed pdl_enter(), i.e. has been resident,
// so it never holds SM slots this grid still needs.  Kernels launched without
// the attribute (or after a copy) find nothing to wait for.
#pragma once
#include <cuda_runtime.h>

namespace gpss {

__device__ __forceinline__ void pdl_enter()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... KArgs, typename... Args>
static cudaError_t launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args... args)
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
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

}  // namespace gpss
