// pdl.cuh -- programmatic dependent launch for chains of short dependent kernels.
#pragma once
#include <cuda_runtime.h>

#include "lmtg_internal.cuh"

namespace lmtg {

// Programmatic dependent launch: a cycle kernel launched with launch_pdl may be scheduled while
// the previous kernel of the stream finishes.  It first waits until that kernel has completed
// and its writes are visible (griddepcontrol.wait, a hardware wait, a no-op without the launch
// attribute), then lets its own successor be scheduled (launch_dependents).  The cycle's coarse
// levels are chains of short dependent launches; this hides part of each launch's latency.
__device__ __forceinline__ void pdl_wait_trigger() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <class... KArgs, class... Args>
inline void launch_pdl(void (*kernel)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t s,
                       Args... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    LMTG_CUDA(cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...));
}

}  // namespace lmtg
