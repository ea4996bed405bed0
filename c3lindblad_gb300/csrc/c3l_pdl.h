// Programmatic dependent launch for the kernels of the graph-replayed steps.
//
// A kernel launched with launch_pdl may start while the kernel before it in
// the stream is still running.  Each such kernel first lets its own
// dependents launch (pdl_launch_dependents), reads only program tables that
// no kernel writes, and then calls pdl_wait() before it reads or writes any
// buffer: griddepcontrol.wait returns once the preceding grid has completed
// and its memory operations are visible (a hardware dependency, not a spin
// loop of this code).  A kernel launched without the attribute, or after a
// non-kernel stream operation, returns from the wait at once.
#pragma once

#include <cuda_runtime.h>

#include <utility>

#include "c3l_gb300.h"

namespace c3l {

__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// kernel<<<grid, block, smem, s>>>(args...), with programmatic stream
// serialization when `pdl` is set; cluster_x > 0 also sets a (cluster_x, 1, 1)
// cluster shape.  Early-launched kernels hold SM resources while they wait, so
// paths that overlap other streams' work (the Arnoldi step beside the shifted
// solves) launch without it.
template <typename... KArgs, typename... Args>
inline c3l_status launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                             unsigned cluster_x, bool pdl, Args&&... args) {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[2];
    unsigned n = 0;
    if (pdl) {
        attr[n].id = cudaLaunchAttributeProgrammaticStreamSerialization;
        attr[n].val.programmaticStreamSerializationAllowed = 1;
        ++n;
    }
    if (cluster_x > 0) {
        attr[n].id = cudaLaunchAttributeClusterDimension;
        attr[n].val.clusterDim.x = cluster_x;
        attr[n].val.clusterDim.y = 1;
        attr[n].val.clusterDim.z = 1;
        ++n;
    }
    cfg.attrs = attr;
    cfg.numAttrs = n;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...) == cudaSuccess ? C3L_OK : C3L_ERR_LAUNCH;
}

}  // namespace c3l
