// Software-pipelined step kernel for the shifted FP32 / BF16 / FP16 storage
// (FP32 collision), for any box: link words for walls and solids, rows of
// any length, no per-cell fields.
//
// Same scheme as the FP64 pipelined kernel (lbm_step_async.cuh): persistent
// warps on tiles of 32 consecutive cells of one x row, one cell per lane;
// while a warp collides tile k, the populations of tile k+1 are already in
// flight as cp.async copies into the warp's two-stage shared-memory buffer.
// cp.async moves 4, 8 or 16 bytes, so each lane copies the aligned 4-byte
// word that holds its element: the element itself for FP32, the word with
// the element in its low or high half for 16-bit storage (the half is kept
// as one bit per direction).  Two lanes may copy the same word; each thread
// reads back only its own copies, so cp.async.wait_group is the only
// synchronisation.  Stores go straight from registers.
//
// AA stays race-free under the prefetch for the reason given in
// lbm_step_async.cuh: the locations a cell reads are the ones it writes.
#pragma once

#include "lbm_step_async.cuh"

namespace lbm {

constexpr int kAsyncLowWarps = 8;

template <int Q>
constexpr size_t async_low_smem_bytes()
{
   return (size_t)kAsyncLowWarps * kAsyncStages * Q * 32 * sizeof(uint32_t);
}

__device__ __forceinline__ void cp_async4(uint32_t smem, const void* g)
{
   asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(smem), "l"(g) : "memory");
}

// Buffers addressed by 32-bit element index slot * plane + cell (the launch
// requires Q * plane < 2^32): a bounced-back direction only changes the
// index, not the base pointer, so no per-direction pointer is selected.
template <typename T>
struct PlanePtrsT {
   const T* src;
   T* dst;
   uint32_t plane;
};

// Raw stored value (S (f - w), as a float) from the copied word.
template <int ST>
__device__ __forceinline__ float word_value(uint32_t w, bool high)
{
   if constexpr (ST == ST_F32) {
      return __uint_as_float(w);
   } else {
      const unsigned short b = (unsigned short)(high ? (w >> 16) : (w & 0xFFFFu));
      if constexpr (ST == ST_F16) return __half2float(__ushort_as_half(b));
      else return __bfloat162float(__ushort_as_bfloat16(b));
   }
}

// Issue the copies of one lane's populations; returns the word-half mask
// (bit s set: direction s sits in the high half of its word).
template <int Q, int ST, int KIND, bool LINKS, bool RAGGED>
__device__ __forceinline__ uint32_t async_issue_low(const PlanePtrsT<typename Store<ST>::T>& pp, const TileLane& tl,
                                                    int lane, uint32_t sbuf)
{
   using T = typename Store<ST>::T;
   uint32_t halves = 0u;
   if ((LINKS || RAGGED) && !tl.active) return halves;
   const uint32_t c = (uint32_t)tl.ci.c;
#pragma unroll
   for (int s = 0; s < Q; s++) {
      const Access a = read_access<Q, KIND, LINKS>(tl.ci, tl.lk, s);
      const uint32_t e = c + (uint32_t)a.off;
      const T* elem = pp.src + ((uint32_t)a.slot * pp.plane + e);
      const void* word = elem;
      if constexpr (sizeof(T) == 2) {
         word = reinterpret_cast<const void*>(reinterpret_cast<uintptr_t>(elem) & ~(uintptr_t)3);
         halves |= (e & 1u) << s;
      }
      cp_async4(sbuf + (uint32_t)(s * 32 + lane) * 4u, word);
   }
   return halves;
}

template <int Q, int ST, int KIND, bool LINKS, bool RAGGED>
__global__ void __launch_bounds__(kAsyncLowWarps * 32) step_async_low_kernel(
   const KParams p, const AsyncGeom ag, const PlanePtrsT<typename Store<ST>::T> pp)
{
   extern __shared__ __align__(16) uint32_t async_low_smem[];
   const int lane = threadIdx.x & 31;
   const int warp = threadIdx.x >> 5;
   const uint32_t nw = gridDim.x * kAsyncLowWarps;
   const uint32_t ntiles = ag.ntiles;
   wait_prior_grid();
   uint32_t* mine = async_low_smem + (size_t)warp * kAsyncStages * Q * 32;
   const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(mine);
   constexpr uint32_t kStageBytes = Q * 32 * 4;
   // tiles: three per warp in a fixed order, then the launch's tile feed
   const bool fed = feed_on(ntiles, nw);
   TileFeed feed{0u, 0u, 1u, false};
   if (fed) feed = feed_start(p.sched, 3u * nw, ntiles, blockIdx.x * kAsyncLowWarps + warp, nw, 1u, lane);
   uint32_t t = blockIdx.x * kAsyncLowWarps + warp;
   if (t < ntiles) {
      uint32_t t1 = t + nw < ntiles ? t + nw : ntiles;
      uint32_t t2 = t + 2u * nw < ntiles ? t + 2u * nw : ntiles;
      TileLane cur;
      tile_lane<LINKS, RAGGED>(p, ag, t, lane, LINKS ? tile_link(p, ag, t, lane) : 0u, cur);
      uint32_t lk_ahead = (LINKS && t1 < ntiles) ? tile_link(p, ag, t1, lane) : 0u;
      uint32_t halves = async_issue_low<Q, ST, KIND, LINKS, RAGGED>(pp, cur, lane, sbase);
      cp_async_commit();
      int stage = 0;
      for (;;) {
         TileLane nxt = cur;
         uint32_t halves_next = 0u;
         if (t1 < ntiles) {
            tile_lane<LINKS, RAGGED>(p, ag, t1, lane, lk_ahead, nxt);
            if (LINKS && t2 < ntiles) lk_ahead = tile_link(p, ag, t2, lane);
            halves_next =
               async_issue_low<Q, ST, KIND, LINKS, RAGGED>(pp, nxt, lane, sbase + (stage ^ 1) * kStageBytes);
         }
         cp_async_commit();
         cp_async_wait_prev();
         if (!(LINKS || RAGGED) || cur.active) {
            float g[Q], o[Q];
            const uint32_t* sm = mine + stage * Q * 32;
#pragma unroll
            for (int s = 0; s < Q; s++) g[s] = word_value<ST>(sm[s * 32 + lane], (halves >> s) & 1u);
            if (p.forced) collide_f32<Q, ST, true>(g, o, p.Ff[0], p.Ff[1], p.Ff[2], 0.0f, p);
            else collide_f32<Q, ST, false>(g, o, 0.0f, 0.0f, 0.0f, 0.0f, p);
            const uint32_t c = (uint32_t)cur.ci.c;
#pragma unroll
            for (int s = 0; s < Q; s++) {
               const Access a = write_access<Q, KIND, LINKS>(cur.ci, cur.lk, s);
               store_raw(pp.dst + ((uint32_t)a.slot * pp.plane + c + (uint32_t)a.off), o[s]);
            }
         }
         if (t1 >= ntiles) break;
         t = t1;
         t1 = t2;
         t2 = feed_after(feed, fed, t2, p.sched, 3u * nw, ntiles, nw, lane);
         cur = nxt;
         halves = halves_next;
         stage ^= 1;
      }
   }
   if (fed) feed_done(p.sched);
}

template <int Q, int ST, int KIND, bool LINKS, bool RAGGED>
cudaError_t launch_async_low(const KParams& p, const AsyncGeom& ag, const void* src, void* dst, cudaStream_t stream)
{
   using T = typename Store<ST>::T;
   // Persistent grid size per device ordinal, set once (the value is the same
   // whichever thread computes it first).
   static std::atomic<int> grid_of_device[64];
   int dev = 0;
   cudaError_t e = cudaGetDevice(&dev);
   if (e != cudaSuccess) return e;
   if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
   auto kern = step_async_low_kernel<Q, ST, KIND, LINKS, RAGGED>;
   constexpr size_t smem = async_low_smem_bytes<Q>();
   int cached = grid_of_device[dev].load(std::memory_order_relaxed);
   if (cached == 0) {
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      int per_sm = 0, nsm = 0;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kAsyncLowWarps * 32, smem);
      if (e != cudaSuccess) return e;
      e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      if (per_sm < 1) return cudaErrorInvalidConfiguration;
      cached = per_sm * nsm;
      grid_of_device[dev].store(cached, std::memory_order_relaxed);
   }
   const uint32_t need = (ag.ntiles + kAsyncLowWarps - 1) / kAsyncLowWarps;
   const unsigned grid = (unsigned)(need < (uint32_t)cached ? need : (uint32_t)cached);
   if ((uint64_t)Q * (uint64_t)p.plane >= (1ull << 32)) return cudaErrorInvalidValue;
   PlanePtrsT<T> pp;
   pp.src = static_cast<const T*>(src);
   pp.dst = static_cast<T*>(dst);
   pp.plane = (uint32_t)p.plane;
   return launch_overlapped(kern, dim3(grid), dim3(kAsyncLowWarps * 32), smem, stream, p, ag, pp);
}

}  // namespace lbm
