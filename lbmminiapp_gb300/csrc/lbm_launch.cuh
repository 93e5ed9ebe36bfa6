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

// Tile order of the persistent step kernels whose tiles differ in cost (link
// words and bounce-back, partial tiles).  Warp w of nw takes its first K tiles
// in a fixed order (w, w + nw, ..., w + (K - 1) nw) and the rest, first = K nw,
// first + 1, ..., from a counter (sched[0], zero at launch) as it asks for
// them, so warps on faster SMs take more tiles and the SMs finish together: a
// fixed round-robin to the end left the last SMs working alone for 5 to 10 %
// of such a step.  (Where every tile costs the same, the fixed order is kept:
// the counter's atomics cost more than they save.)  Lane 0 asks one tile
// ahead, so the atomic's latency hides behind a tile of work.  A warp keeps
// calling feed_next() until it returns ntiles; every thread of the block then
// calls feed_done(), and the last block to get there sets both counter words
// back to zero for the next launch.  All calls are warp-uniform and come after
// wait_prior_grid().
struct TileFeed {
   uint32_t pend;   // lane 0: the counter value of the next dynamic tile
   bool more;
};

__device__ __forceinline__ TileFeed feed_start(uint32_t* sched, uint32_t first, uint32_t ntiles, int lane)
{
   TileFeed f{0u, first < ntiles};
   if (f.more && lane == 0) f.pend = atomicAdd(sched, 1u);
   return f;
}

// The next dynamic tile, ntiles when none is left.
__device__ __forceinline__ uint32_t feed_next(TileFeed& f, uint32_t* sched, uint32_t first, uint32_t ntiles,
                                              int lane)
{
   if (!f.more) return ntiles;
   const uint32_t v = __shfl_sync(0xFFFFFFFFu, f.pend, 0);
   if (v >= ntiles - first) {
      f.more = false;
      return ntiles;
   }
   if (lane == 0) f.pend = atomicAdd(sched, 1u);
   return first + v;
}

__device__ __forceinline__ void feed_done(uint32_t* sched)
{
   __syncthreads();
   if (threadIdx.x != 0) return;
   __threadfence();
   if (atomicAdd(sched + 1, 1u) == gridDim.x - 1u) {
      atomicExch(sched, 0u);
      atomicExch(sched + 1, 0u);
   }
}

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
