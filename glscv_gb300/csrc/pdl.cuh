// pdl.cuh -- programmatic dependent launch: the kernel-side entry and the
// host-side launch with the attribute.
#pragma once
#include <cuda_runtime.h>

#include <utility>

namespace glsfft {

// A grid launched with the programmatic-serialisation attribute can be made
// resident while its stream predecessor is still running; it waits here,
// before its first global access, until that grid has completed and its
// memory is visible, then lets its own successor launch.  Both instructions
// return at once in a grid launched without the attribute.
__device__ __forceinline__ void pdl_enter() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launch `kern` with the attribute when `pdl` is set (the kernel must begin
// with pdl_enter()), else as an ordinary launch.
template <typename... KArgs, typename... Args>
inline cudaError_t launch_maybe_pdl(bool pdl, void (*kern)(KArgs...), dim3 grid, dim3 block,
                                    size_t smem, cudaStream_t s, Args &&...args) {
    if (!pdl) {
        kern<<<grid, block, smem, s>>>(std::forward<Args>(args)...);
        return cudaGetLastError();
    }
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

}  // namespace glsfft
