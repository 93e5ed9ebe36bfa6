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

// Tile order of the persistent step kernels.  Warp w of nw takes its first K
// tiles in a fixed order (w, w + nw, ..., w + (K - 1) nw) and, when the launch
// has at least kFeedMinTiles tiles per warp, the rest as it asks for them, so
// warps on faster SMs take more tiles and the SMs finish together: a fixed
// round-robin to the end left the last SMs working alone for 3 to 10 % of a
// step, and let the warps drift apart far enough to lose the L2 reuse between
// neighbouring rows.  (With fewer tiles per warp the fixed order continues to
// the end: the feed's atomics would cost more than they save.)  The tiles
// past first = K nw are dealt to ng = min(groups, nw) groups in interleaved
// chunks of kFeedChunk consecutive tiles (chunk q of group g starts at
// first + (q ng + g) kFeedChunk), each group with its own counter, which warp
// w draws from for g = w mod ng.  A kernel that takes many small tiles (the compact
// odd step, about 0.7 G tiles/s) made a single counter's address the
// bottleneck; for the others one counter keeps neighbouring tiles together
// and runs faster.  Lane 0 asks one tile ahead, so the atomic's
// latency hides behind a tile of work.  A warp keeps calling feed_next() until
// it returns ntiles; every thread of the block then calls feed_done(), and the
// last block to get there sets the counters back to zero for the next launch.
// All calls are warp-uniform and come after wait_prior_grid().
constexpr uint32_t kFeedMinTiles = 16;
constexpr uint32_t kFeedGroups = 8;
constexpr uint32_t kFeedChunk = 32;
constexpr uint32_t kFeedStride = 32;                                   // words: one 128-byte line per counter
constexpr uint32_t kFeedWords = (kFeedGroups + 1) * kFeedStride;       // the counters and the finished-block count

struct TileFeed {
   uint32_t pend;   // lane 0: the group counter's value for the next dynamic tile
   uint32_t g;      // the warp's group
   uint32_t ng;     // groups: kFeedGroups, fewer when the grid has fewer warps
   bool more;
};

// groups: 1 to kFeedGroups counters (more for kernels that take many small tiles)
__device__ __forceinline__ TileFeed feed_start(uint32_t* sched, uint32_t first, uint32_t ntiles, uint32_t w,
                                               uint32_t nw, uint32_t groups, int lane)
{
   const uint32_t ng = nw < groups ? nw : groups;
   TileFeed f{0u, w % ng, ng, (uint64_t)first + (uint64_t)(w % ng) * kFeedChunk < ntiles};
   if (f.more && lane == 0) f.pend = atomicAdd(sched + f.g * kFeedStride, 1u);
   return f;
}

// The next dynamic tile, ntiles when none is left (a group's tiles rise with
// its counter, so once one is past the end all later ones are).
__device__ __forceinline__ uint32_t feed_next(TileFeed& f, uint32_t* sched, uint32_t first, uint32_t ntiles,
                                              int lane)
{
   if (!f.more) return ntiles;
   const uint32_t v = __shfl_sync(0xFFFFFFFFu, f.pend, 0);
   const uint64_t t = (uint64_t)first + ((uint64_t)(v / kFeedChunk) * f.ng + f.g) * kFeedChunk + v % kFeedChunk;
   if (t >= ntiles) {
      f.more = false;
      return ntiles;
   }
   if (lane == 0) f.pend = atomicAdd(sched + f.g * kFeedStride, 1u);
   return (uint32_t)t;
}

// Whether a launch of ntiles tiles over nw warps takes its tiles from the feed.
__device__ __forceinline__ bool feed_on(uint32_t ntiles, uint32_t nw)
{
   return (uint64_t)ntiles >= (uint64_t)kFeedMinTiles * nw;
}

// The warp's tile after `last` (the latest it holds, or ntiles): from the feed
// when it is on, else the next one of the fixed order.
__device__ __forceinline__ uint32_t feed_after(TileFeed& f, bool on, uint32_t last, uint32_t* sched, uint32_t first,
                                               uint32_t ntiles, uint32_t nw, int lane)
{
   if (last >= ntiles) return ntiles;
   if (on) return feed_next(f, sched, first, ntiles, lane);
   return last + nw < ntiles ? last + nw : ntiles;
}

__device__ __forceinline__ void feed_done(uint32_t* sched)
{
   __syncthreads();
   if (threadIdx.x != 0) return;
   __threadfence();
   if (atomicAdd(sched + kFeedGroups * kFeedStride, 1u) == gridDim.x - 1u) {
      for (uint32_t g = 0; g <= kFeedGroups; g++) atomicExch(sched + g * kFeedStride, 0u);
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
