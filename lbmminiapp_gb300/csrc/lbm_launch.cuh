// Overlapped launches of the step kernels.
//
// A step kernel is launched with programmatic stream serialisation: the
// driver may schedule its blocks while the previous kernel on the stream is
// still draining (the persistent grids' last tiles, or the launch latency of
// a short step on a small box).  Each step kernel calls wait_prior_grid()
// before its first global-memory access, which returns once the previous
// grid has completed and its writes are visible, so the in-place AA steps
// and everything else on the stream keep their order.  In a normal launch the
// wait returns at once.
#pragma once

#include <cuda_runtime.h>

#include <utility>

namespace lbm {

__device__ __forceinline__ void wait_prior_grid() { asm volatile("griddepcontrol.wait;\n" ::: "memory"); }

template <typename... KArgs, typename... Args>
cudaError_t launch_overlapped(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                              Args&&... args)
{
   cudaLaunchConfig_t cfg = {};
   cfg.gridDim = grid;
   cfg.blockDim = block;
   cfg.dynamicSmemBytes = smem;
   cfg.stream = stream;
   cudaLaunchAttribute attr[1];
   attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
   attr[0].val.programmaticStreamSerializationAllowed = 1;
   cfg.attrs = attr;
   cfg.numAttrs = 1;
   return cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

}  // namespace lbm
