// Software-pipelined step kernel for FP64 storage with F64X arithmetic (any
// box; link words for walls and solids; no per-cell fields).
//
// The F64X collision is about 1.7k instructions per cell, so the plain
// one-cell-per-thread kernel spends its time either issuing or waiting on its
// 19/27 loads with only 16 warps per SM resident (128 registers per thread).
// Here every warp is persistent and works on tiles of 32 consecutive cells of
// one x row: while it collides tile k it already has the loads of tile k+1 in
// flight as cp.async copies (8 bytes per thread and direction) into its own
// two-stage shared-memory buffer, so the loads hold no registers and their
// latency overlaps the collision.  Each thread reads back only what it copied
// itself, so cp.async.wait_group is the only synchronisation needed.
//
// AA (in place) stays race-free under the prefetch: the locations a cell's
// thread reads are exactly the ones it writes (even step: its own slots; odd
// step: slot s at x - c_s and slot opp(s) at x + c_s form the same set, a
// bounced-back direction reading and writing the own cell), so a
// prefetch of another tile never sees a write of this one.
#pragma once

#include <atomic>

#include "lbm_launch.cuh"
#include "lbm_step.cuh"

namespace lbm {

// Warps per block and blocks per SM, measured on GB300: D3Q19 steps run best
// with 8-warp blocks, two per SM (128 registers), D3Q27 steps with 4-warp
// blocks, three per SM (at most 170 registers; at 128 they spill and run
// 15-20 % slower).
template <int Q, int KIND>
constexpr int async_warps() { return Q == 19 ? 8 : 4; }
template <int Q, int KIND>
constexpr int async_min_blocks() { return async_warps<Q, KIND>() == 8 ? 2 : 3; }
constexpr int kAsyncStages = 2;

template <int Q, int KIND>
constexpr size_t async_smem_bytes()
{
   return (size_t)async_warps<Q, KIND>() * kAsyncStages * Q * 32 * sizeof(unsigned long long);
}

// Tiles of 32 cells: tile t covers x in [32 (t mod ntx), +32) of row t / ntx,
// row r = y + ny z, with ntx = ceil(nx / 32) (lanes past the row end idle).  Divisions by a run-time d use q = umulhi64(n, m) with
// m = ceil(2^64 / d) (exact for n, d < 2^32); d = 1 is m = 0.
struct AsyncGeom {
   uint32_t ntiles, ntx;
   uint64_t m_ntx, m_ny;
};

__device__ __forceinline__ uint32_t div_magic(uint32_t n, uint32_t d, uint64_t m)
{
   return m ? (uint32_t)__umul64hi((uint64_t)n, m) : n;
}

// Returns false for a lane past the end of its row.
__device__ __forceinline__ bool tile_cell(const KParams& p, const AsyncGeom& ag, uint32_t t, int lane,
                                          CellIndex& ci)
{
   const uint32_t row = div_magic(t, ag.ntx, ag.m_ntx);
   const int x = (int)(t - row * ag.ntx) * 32 + lane;
   const uint32_t z = div_magic(row, (uint32_t)p.ny, ag.m_ny);
   const int y = (int)(row - z * (uint32_t)p.ny);
   ci.c = (int64_t)row * p.nx + x;
   ci.dxm = (x == 0) ? p.nx - 1 : -1;
   ci.dxp = (x == p.nx - 1) ? -(p.nx - 1) : 1;
   ci.dym = (y == 0) ? (p.ny - 1) * p.nx : -p.nx;
   ci.dyp = (y == p.ny - 1) ? -(p.ny - 1) * p.nx : p.nx;
   const int nxy = p.nx * p.ny;
   ci.dzm = (z == 0) ? (p.nz - 1) * nxy : -nxy;
   ci.dzp = ((int)z == p.nz - 1) ? -(p.nz - 1) * nxy : nxy;
   return x < p.nx;
}

__device__ __forceinline__ void cp_async8(uint32_t smem, const void* g)
{
   asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(smem), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;\n" ::: "memory"); }

// Base pointer of every direction plane of the source and target buffers,
// passed by value so each sits in the kernel's parameter bank: an access is
// then one wide multiply-add of a 32-bit cell index (fewer than 2^31 cells;
// the periodic wrap keeps neighbour indices inside the box) onto a
// parameter-bank pointer.
struct PlanePtrs {
   const unsigned long long* src[27];
   unsigned long long* dst[27];
};

// Lane state of a tile: its cell, its link word (0 without walls) and
// whether it updates anything (inside the row, not solid).
struct TileLane {
   CellIndex ci;
   uint32_t lk;
   bool active;
};

// Link word of this lane's cell in tile t (the solid bit past the row end).
__device__ __forceinline__ uint32_t tile_link(const KParams& p, const AsyncGeom& ag, uint32_t t, int lane)
{
   const uint32_t row = div_magic(t, ag.ntx, ag.m_ntx);
   const int x = (int)(t - row * ag.ntx) * 32 + lane;
   return x < p.nx ? __ldg(p.links + (int64_t)row * p.nx + x) : kSolidBit;
}

// lk: the tile's link words, loaded one tile ahead so the load's latency
// hides behind a collision.
// RAGGED: nx is not a multiple of 32, so some lanes fall past their row.
template <bool LINKS, bool RAGGED>
__device__ __forceinline__ void tile_lane(const KParams& p, const AsyncGeom& ag, uint32_t t, int lane, uint32_t lk,
                                          TileLane& tl)
{
   const bool inside = tile_cell(p, ag, t, lane, tl.ci);
   tl.active = RAGGED ? inside : true;
   tl.lk = LINKS ? lk : 0u;
   if (LINKS) tl.active = tl.active && !(lk & kSolidBit);
}

template <int Q, int KIND, bool LINKS, bool RAGGED>
__device__ __forceinline__ void async_issue(const PlanePtrs& pp, const TileLane& tl, int lane, uint32_t sbuf)
{
   if ((LINKS || RAGGED) && !tl.active) return;
   const uint32_t c = (uint32_t)tl.ci.c;
#pragma unroll
   for (int s = 0; s < Q; s++) {
      const Access a = read_access<Q, KIND, LINKS>(tl.ci, tl.lk, s);
      cp_async8(sbuf + (uint32_t)(s * 32 + lane) * 8u, pp.src[a.slot] + (c + (uint32_t)a.off));
   }
}

// Stores each output straight to its target slot.  AA stays race-free with
// stores that may be overwritten later by the same thread (the fast path's
// outputs when a range check fails): the locations are this cell's own.
template <int Q, int KIND, bool LINKS>
struct StoreEmit {
   const PlanePtrs& pp;
   const CellIndex& ci;
   uint32_t lk;
   __device__ __forceinline__ void operator()(int s, uint64_t v) const
   {
      const Access a = write_access<Q, KIND, LINKS>(ci, lk, s);
      pp.dst[a.slot][(uint32_t)ci.c + (uint32_t)a.off] = v;
   }
   // A non-rest direction s known at run time, with o = opp(s) and c_s.
   __device__ __forceinline__ void put(int s, int o, int cx, int cy, int cz, uint64_t v) const
   {
      const Access a = write_access_rt<KIND, LINKS>(ci, lk, s, o, cx, cy, cz);
      pp.dst[a.slot][(uint32_t)ci.c + (uint32_t)a.off] = v;
   }
};

template <int Q, int KIND, bool LINKS, bool RAGGED>
__global__ void __launch_bounds__(async_warps<Q, KIND>() * 32, async_min_blocks<Q, KIND>()) step_async_kernel(const KParams p, const AsyncGeom ag,
                                                                      const PlanePtrs pp)
{
   extern __shared__ __align__(16) unsigned long long async_smem[];
   const int lane = threadIdx.x & 31;
   const int warp = threadIdx.x >> 5;
   constexpr int kWarps = async_warps<Q, KIND>();
   const uint32_t nw = gridDim.x * kWarps;
   const uint32_t ntiles = ag.ntiles;
   wait_prior_grid();
   unsigned long long* mine = async_smem + (size_t)warp * kAsyncStages * Q * 32;
   const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(mine);
   constexpr uint32_t kStageBytes = Q * 32 * 8;
   // tiles: three per warp in a fixed order, then the launch's tile feed (8
   // counters for the D3Q19 tiles, which it hands out fastest); t is collided
   // while t1's populations are in flight and t2's link words are loaded
   const bool fed = feed_on(ntiles, nw);
   TileFeed feed{0u, 0u, 1u, false};
   if (fed) feed = feed_start(p.sched, 3u * nw, ntiles, blockIdx.x * kWarps + warp, nw, Q == 19 ? kFeedGroups : 1u, lane);
   uint32_t t = blockIdx.x * kWarps + warp;
   if (t < ntiles) {
      uint32_t t1 = t + nw < ntiles ? t + nw : ntiles;
      uint32_t t2 = t + 2u * nw < ntiles ? t + 2u * nw : ntiles;
      TileLane cur;
      tile_lane<LINKS, RAGGED>(p, ag, t, lane, LINKS ? tile_link(p, ag, t, lane) : 0u, cur);
      uint32_t lk_ahead = (LINKS && t1 < ntiles) ? tile_link(p, ag, t1, lane) : 0u;
      async_issue<Q, KIND, LINKS, RAGGED>(pp, cur, lane, sbase);
      cp_async_commit();
      int stage = 0;
      for (;;) {
         TileLane nxt = cur;
         if (t1 < ntiles) {
            tile_lane<LINKS, RAGGED>(p, ag, t1, lane, lk_ahead, nxt);
            if (LINKS && t2 < ntiles) lk_ahead = tile_link(p, ag, t2, lane);
            async_issue<Q, KIND, LINKS, RAGGED>(pp, nxt, lane, sbase + (stage ^ 1) * kStageBytes);
         }
         cp_async_commit();
         cp_async_wait_prev();
         if (!(LINKS || RAGGED) || cur.active) {
            // each output is stored as the collision makes it, and the update
            // re-reads its inputs from shared memory: neither the Q input nor the
            // Q output patterns stay in registers
            // D3Q27 AB pull (stores to the cell's own slots) runs the pair-class
            // loops: 9.69 -> 9.96 GLUPS on the 256x128x128 channel.  Where the
            // stores go to neighbours (AB push: 9.92 -> 9.12) each store's
            // offset would cost more than the smaller code saves.
            StoreEmit<Q, KIND, LINKS> emit{pp, cur.ci, cur.lk};
            collide_f64x_shared_emit<Q, Q == 27 && KIND == K_AB_PULL>(mine + stage * Q * 32 + lane, p, emit);
         }
         if (t1 >= ntiles) break;
         t = t1;
         t1 = t2;
         t2 = feed_after(feed, fed, t2, p.sched, 3u * nw, ntiles, nw, lane);
         cur = nxt;
         stage ^= 1;
      }
   }
   if (fed) feed_done(p.sched);
}

inline AsyncGeom async_geom(int nx, int ny, int nz)
{
   AsyncGeom g;
   g.ntx = (uint32_t)((nx + 31) / 32);
   g.ntiles = g.ntx * (uint32_t)ny * (uint32_t)nz;
   g.m_ntx = g.ntx == 1 ? 0 : (~0ull / g.ntx) + 1;
   g.m_ny = ny == 1 ? 0 : (~0ull / (uint64_t)ny) + 1;
   return g;
}

// Persistent grid: as many blocks as fit on the device at once (queried once
// per device and kernel; the shared-memory opt-in is set at the same time).
template <int Q, int KIND, bool LINKS, bool RAGGED>
cudaError_t launch_async(const KParams& p, const AsyncGeom& ag, const void* src, void* dst, cudaStream_t stream)
{
   // Persistent grid size per device ordinal, set once (the value is the same
   // whichever thread computes it first).
   static std::atomic<int> grid_of_device[64];
   int dev = 0;
   cudaError_t e = cudaGetDevice(&dev);
   if (e != cudaSuccess) return e;
   if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
   auto kern = step_async_kernel<Q, KIND, LINKS, RAGGED>;
   constexpr int kWarps = async_warps<Q, KIND>();
   constexpr size_t smem = async_smem_bytes<Q, KIND>();
   int cached = grid_of_device[dev].load(std::memory_order_relaxed);
   if (cached == 0) {
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      int per_sm = 0, nsm = 0;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kWarps * 32, smem);
      if (e != cudaSuccess) return e;
      e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      if (per_sm < 1) return cudaErrorInvalidConfiguration;
      cached = per_sm * nsm;
      grid_of_device[dev].store(cached, std::memory_order_relaxed);
   }
   const uint32_t need = (ag.ntiles + kWarps - 1) / kWarps;
   const unsigned grid = (unsigned)(need < (uint32_t)cached ? need : (uint32_t)cached);
   PlanePtrs pp;
   for (int s = 0; s < 27; s++) {
      const int k = s < Q ? s : 0;
      pp.src[s] = static_cast<const unsigned long long*>(src) + (int64_t)k * p.plane;
      pp.dst[s] = static_cast<unsigned long long*>(dst) + (int64_t)k * p.plane;
   }
   return launch_overlapped(kern, dim3(grid), dim3(kWarps * 32), smem, stream, p, ag, pp);
}

}  // namespace lbm
