// AA step kernels on the compact fluid-only layout (lbm_compact.cuh) for the
// shifted FP32 / BF16 / FP16 storage with FP32 collision, and the copies
// between the compact and the dense layouts.
//
// Both steps use the pipelined scheme of the dense kernels
// (lbm_step_async_low.cuh): persistent warps, and the populations of the next
// tile in flight as cp.async copies into a two-stage shared buffer per warp
// while the current tile collides.  No lane holds a solid cell, and every
// sector moved holds fluid populations only.  Tiles come from the tile feed
// (lbm_launch.cuh): a fixed first round, then counters.
//
//   even step (KernelAA_SOA_Base.cpp:173-254): tiles of 64 consecutive fluid
//     indices, two cells per lane; read own slot opp(s), write own slot s, one
//     aligned word per slot for both cells: contiguous accesses.
//   odd step (KernelAA_SOA_Base.cpp:257-342): row tiles of up to 32 fluid
//     cells, one per lane, so the 9 neighbour rows are the same for the whole
//     warp; read slot s at x - c_s (own slot opp(s) when that neighbour is
//     blocked), write slot opp(s) at x + c_s (own slot s when blocked).  Each
//     lane copies the 4-byte word holding each of its elements; the tile's
//     metadata is copied two tiles ahead.
//
// AA stays race-free under the prefetch and in any tile order for the dense
// layout's reason: a cell's reads and writes touch the same set of elements,
// so a prefetch of another tile never reads an element this tile writes.  A
// copied word may hold a second element written by another cell; only the
// lane's own half is used.
#include <atomic>

#include "lbm_compact.cuh"
#include "lbm_launch.cuh"
#include "lbm_step_async_low.cuh"

namespace lbm {
namespace {

constexpr int kCompactWarps = 8;

// Two consecutive stored elements as one word: the even step's copy unit.
template <typename T> struct PairWord;
template <> struct PairWord<float> {
   using W = uint2;
   __device__ static void unpack(W w, float& a, float& b) { a = __uint_as_float(w.x); b = __uint_as_float(w.y); }
   __device__ static W pack(float a, float b) { return make_uint2(__float_as_uint(a), __float_as_uint(b)); }
};
template <> struct PairWord<__half> {
   using W = uint32_t;
   __device__ static void unpack(W w, float& a, float& b)
   {
      const float2 f = __half22float2(*reinterpret_cast<const __half2*>(&w));
      a = f.x;
      b = f.y;
   }
   __device__ static W pack(float a, float b)
   {
      const __half2 h = __floats2half2_rn(a, b);
      return *reinterpret_cast<const uint32_t*>(&h);
   }
};
template <> struct PairWord<__nv_bfloat16> {
   using W = uint32_t;
   __device__ static void unpack(W w, float& a, float& b)
   {
      const float2 f = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&w));
      a = f.x;
      b = f.y;
   }
   __device__ static W pack(float a, float b)
   {
      const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
      return *reinterpret_cast<const uint32_t*>(&h);
   }
};

// Per warp, the odd step's pipeline: while tile j collides, tile j + 1's
// populations and tile j + 2's metadata are copied: two population stages and
// three metadata slots, each slot the tile record, the lanes' row counts and
// the lanes' link words.
constexpr uint32_t kOddStages = 2;
constexpr uint32_t kMetaSlots = 3;
constexpr uint32_t kMetaTile = 0;                         // OddTile, 20 words
constexpr uint32_t kMetaU = 20;                           // uint2 per lane
constexpr uint32_t kMetaLk = kMetaU + 2 * 32;             // uint32 per lane
constexpr uint32_t kMetaWords = kMetaLk + 32;             // 116 words, 464 bytes
static_assert(kMetaWords % 4 == 0, "metadata slots stay 16-byte aligned");

// Words of shared memory per warp of the odd step: the population stages
// (one word per lane and direction) and the metadata slots.
template <int Q>
constexpr uint32_t odd_warp_words() { return kOddStages * Q * 32 + kMetaSlots * kMetaWords; }

// Shared memory per block: a two-stage buffer per warp of one word per lane
// and direction (the even step's words hold two cells), and the odd step's
// metadata slots.
template <int Q, int ST, int KIND>
constexpr size_t compact_smem_bytes()
{
   using T = typename Store<ST>::T;
   return KIND == K_AA_EVEN ? (size_t)kCompactWarps * kAsyncStages * Q * 32 * sizeof(typename PairWord<T>::W)
                            : (size_t)kCompactWarps * odd_warp_words<Q>() * sizeof(uint32_t);
}

// Address of the aligned 4-byte word holding element e (the element itself
// for 4-byte storage).
template <typename T>
__device__ __forceinline__ const void* word_of(const T* base, uint32_t e)
{
   if constexpr (sizeof(T) == 2)
      return reinterpret_cast<const void*>(reinterpret_cast<uintptr_t>(base + e) & ~(uintptr_t)3);
   else
      return base + e;
}

template <int Q, int ST, bool FORCE>
__device__ __forceinline__ void collide_cell(const float (&G)[Q], float (&o)[Q], const KParams& p)
{
   if (FORCE) collide_f32<Q, ST, true>(G, o, p.Ff[0], p.Ff[1], p.Ff[2], 0.0f, p);
   else collide_f32<Q, ST, false>(G, o, 0.0f, 0.0f, 0.0f, 0.0f, p);
}

// ------------------------------------------------------------------ even
// Two cells per lane: tiles of 64 consecutive fluid indices, lane l takes
// cells i0 = 64 t + 2 l and i0 + 1, whose slot-s elements form one aligned
// word (i0 and the slot offsets are even).  A tail pair past nf runs on the
// plane padding (cplane > nf, zero-filled), which no fluid cell reads.
template <int Q, int ST, bool FORCE>
__global__ void __launch_bounds__(kCompactWarps * 32, 2) compact_even_kernel(const KParams p, const CompactGeom g,
                                                                             typename Store<ST>::T* buf)
{
   using T = typename Store<ST>::T;
   using PW = PairWord<T>;
   using W = typename PW::W;
   extern __shared__ __align__(16) uint32_t compact_smem[];
   const int lane = threadIdx.x & 31;
   const int warp = threadIdx.x >> 5;
   const uint32_t ntiles = (g.nf + 63) / 64;
   const uint32_t nw = gridDim.x * kCompactWarps;
   wait_prior_grid();
   W* mine = reinterpret_cast<W*>(compact_smem) + (size_t)warp * kAsyncStages * Q * 32;
   const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(mine);
   constexpr uint32_t kStageBytes = Q * 32 * sizeof(W);
   auto issue = [&](uint32_t tt, uint32_t sb) {
      const uint32_t i0 = tt * 64 + 2 * (uint32_t)lane;
      if (i0 >= g.nf) return;
#pragma unroll
      for (int s = 0; s < Q; s++) {
         const uint32_t dst = sb + (uint32_t)(s * 32 + lane) * (uint32_t)sizeof(W);
         const T* src = buf + (g.soff[lat_opp(Q, s)] + i0);
         if constexpr (sizeof(W) == 8) cp_async8(dst, src);
         else cp_async4(dst, src);
      }
   };
   // tiles: two per warp in a fixed order, then the launch's tile feed
   const bool fed = feed_on(ntiles, nw);
   TileFeed feed{0u, 0u, 1u, false};
   if (fed) feed = feed_start(p.sched, 2u * nw, ntiles, blockIdx.x * kCompactWarps + warp, nw, 1u, lane);
   uint32_t t = blockIdx.x * kCompactWarps + warp;
   if (t < ntiles) {
      uint32_t t1 = t + nw < ntiles ? t + nw : ntiles;
      issue(t, sbase);
      cp_async_commit();
      int stage = 0;
      for (;;) {
         if (t1 < ntiles) issue(t1, sbase + (stage ^ 1) * kStageBytes);
         cp_async_commit();
         cp_async_wait_prev();
         const uint32_t i0 = t * 64 + 2 * (uint32_t)lane;
         if (i0 < g.nf) {
            const W* sm = mine + stage * Q * 32;
            float G0[Q], G1[Q];
#pragma unroll
            for (int s = 0; s < Q; s++) PW::unpack(sm[s * 32 + lane], G0[s], G1[s]);
            auto emit = [&](int s, float a, float b) {
               *reinterpret_cast<W*>(buf + (g.soff[s] + i0)) = PW::pack(a, b);
            };
            collide2_f32_emit<Q, ST, FORCE>(G0, G1, p, emit);
         }
         if (t1 >= ntiles) break;
         t = t1;
         t1 = feed_after(feed, fed, t1, p.sched, 2u * nw, ntiles, nw, lane);
         stage ^= 1;
      }
   }
   if (fed) feed_done(p.sched);
}

// ------------------------------------------------------------------ odd
__device__ __forceinline__ void cp_async16(uint32_t smem, const void* g)
{
   asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(smem), "l"(g) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

// Copies tile t's metadata into a slot (sm: its shared-memory address).
__device__ __forceinline__ void odd_meta_issue(const CompactGeom& g, uint32_t t, int lane, uint32_t sm)
{
   if (lane < 5) cp_async16(sm + 4u * kMetaTile + 16u * lane, reinterpret_cast<const uint4*>(g.tiles + t) + lane);
   const uint32_t tl = t * 32u + (uint32_t)lane;
   cp_async8(sm + 4u * kMetaU + 8u * lane, g.u + tl);
   cp_async4(sm + 4u * kMetaLk + 4u * lane, g.lk + tl);
}

// A lane's view of its tile: its cell i, link word, and the compact index of
// the fluid cell at x (N), one below (Nm: at x - 1) and one past (Np: at x + 1)
// in each row k, valid where that neighbour is fluid.
template <int Q>
struct OddView {
   uint32_t i, lk;
   uint32_t N[9], Nm[9], Np[9];
};

// Direction index of the velocity (cx, cy, cz), -1 if the lattice has none.
__host__ __device__ constexpr int dir_of(int Q, int cx, int cy, int cz)
{
   for (int s = 0; s < Q; s++)
      if (lat_c(Q, s, 0) == cx && lat_c(Q, s, 1) == cy && lat_c(Q, s, 2) == cz) return s;
   return -1;
}

template <int Q>
__device__ __forceinline__ void odd_view(const uint32_t* m, int lane, OddView<Q>& v)
{
   v.lk = m[kMetaLk + lane];
   const uint2 u = *reinterpret_cast<const uint2*>(m + kMetaU + 2 * lane);
   const uint4 b0 = *reinterpret_cast<const uint4*>(m + kMetaTile);
   const uint4 b1 = *reinterpret_cast<const uint4*>(m + kMetaTile + 4);
   const uint32_t b[9] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w, m[kMetaTile + 8]};
   v.i = b[4] + (uint32_t)lane;
#pragma unroll
   for (int k = 0; k < 9; k++) {
      if (k == 4) {
         v.N[4] = v.i;
         v.Nm[4] = v.i - 1u;
         v.Np[4] = v.i + 1u;
         continue;
      }
      const int byte = k < 4 ? k : k - 1;
      const uint32_t w = byte < 4 ? u.x : u.y;
      v.N[k] = b[k] + __byte_perm(w, 0u, 0x4440u | (uint32_t)(byte & 3));
      v.Nm[k] = v.N[k] - 1u;
      // one past (x, row k) when that cell is fluid: the link bit of (0, dy, dz)
      v.Np[k] = v.N[k] + (((v.lk >> dir_of(Q, 0, k / 3 - 1, k % 3 - 1)) & 1u) ^ 1u);
   }
   if (v.lk & (kRowStartBit | kRowEndBit)) {
      // a row end: the periodic wrap of x
      const uint32_t* n = m + kMetaTile + 9;
#pragma unroll
      for (int k = 0; k < 9; k++) {
         if (v.lk & kRowStartBit) v.Nm[k] += n[k];
         if (v.lk & kRowEndBit) v.Np[k] -= n[k];
      }
   }
}

// Element of the fluid neighbour at x + (dx, dy, dz), slot offset excluded.
template <int Q>
__device__ __forceinline__ uint32_t odd_nbr(const OddView<Q>& v, int dx, int dy, int dz)
{
   const int k = (dy + 1) * 3 + (dz + 1);
   return dx == 0 ? v.N[k] : (dx < 0 ? v.Nm[k] : v.Np[k]);
}

// Element e_s read for direction opp(s) and written for direction s: slot
// opp(s) of the neighbour at x + c_s, own slot s when that neighbour is
// blocked (and for the rest direction).
template <int Q>
__device__ __forceinline__ uint32_t odd_elem(const CompactGeom& g, const OddView<Q>& v, int s)
{
   if (s == lat_rest(Q) || ((v.lk >> s) & 1u)) return g.soff[s] + v.i;
   return g.soff[lat_opp(Q, s)] + odd_nbr<Q>(v, lat_c(Q, s, 0), lat_c(Q, s, 1), lat_c(Q, s, 2));
}

// Copies the lane's populations (direction s from e_opp(s)); returns the
// word-half mask.
template <int Q, typename T>
__device__ __forceinline__ uint32_t odd_pop_issue(const T* buf, const CompactGeom& g, const OddView<Q>& v, int lane,
                                                  uint32_t sb)
{
   uint32_t halves = 0u;
#pragma unroll
   for (int s = 0; s < Q; s++) {
      const uint32_t e = odd_elem<Q>(g, v, lat_opp(Q, s));
      cp_async4(sb + (uint32_t)(s * 32 + lane) * 4u, word_of(buf, e));
      if constexpr (sizeof(T) == 2) halves |= (e & 1u) << s;
   }
   return halves;
}

// Tiles: three per warp in a fixed order, the rest from the launch's tile
// feed (lbm_launch.cuh) with 8 counters (tiles differ in cost: bounce-back,
// partial tiles; and they are small, so one counter would be the bottleneck).
template <int Q, int ST, bool FORCE>
__global__ void __launch_bounds__(kCompactWarps * 32, 2) compact_odd_kernel(const KParams p, const CompactGeom g,
                                                                            typename Store<ST>::T* buf)
{
   extern __shared__ __align__(16) uint32_t compact_smem[];
   const int lane = threadIdx.x & 31;
   const int warp = threadIdx.x >> 5;
   const uint32_t ntiles = g.nrow_tiles;
   const uint32_t nw = gridDim.x * kCompactWarps;
   wait_prior_grid();
   uint32_t* pop = compact_smem + (size_t)warp * odd_warp_words<Q>();
   uint32_t* meta = pop + kOddStages * Q * 32;
   const uint32_t pop_s = (uint32_t)__cvta_generic_to_shared(pop);
   const uint32_t meta_s = (uint32_t)__cvta_generic_to_shared(meta);
   constexpr uint32_t kStageBytes = Q * 32 * 4;
   constexpr uint32_t kSlotBytes = kMetaWords * 4;
   const bool fed = feed_on(ntiles, nw);
   TileFeed feed{0u, 0u, 1u, false};
   if (fed) feed = feed_start(p.sched, 3u * nw, ntiles, blockIdx.x * kCompactWarps + warp, nw, kFeedGroups, lane);
   uint32_t t = blockIdx.x * kCompactWarps + warp;
   if (t < ntiles) {
      uint32_t t1 = t + nw < ntiles ? t + nw : ntiles;
      uint32_t t2 = t + 2u * nw < ntiles ? t + 2u * nw : ntiles;
      odd_meta_issue(g, t, lane, meta_s);
      if (t1 < ntiles) odd_meta_issue(g, t1, lane, meta_s + kSlotBytes);
      cp_async_commit();
      cp_async_wait_all();
      __syncwarp();
      uint32_t halves = 0u;
      {
         OddView<Q> v;
         odd_view<Q>(meta, lane, v);
         if (!(v.lk & kSolidBit)) halves = odd_pop_issue<Q>(buf, g, v, lane, pop_s);
      }
      cp_async_commit();
      uint32_t slot = 0, stage = 0;
      for (;;) {
         const uint32_t slot1 = slot == 2 ? 0 : slot + 1, slot2 = slot1 == 2 ? 0 : slot1 + 1;
         const uint32_t t3 = feed_after(feed, fed, t2, p.sched, 3u * nw, ntiles, nw, lane);
         // this tile's populations and the next tile's metadata have landed
         cp_async_wait_all();
         __syncwarp();
         if (t2 < ntiles) odd_meta_issue(g, t2, lane, meta_s + slot2 * kSlotBytes);
         uint32_t halves_next = 0u;
         if (t1 < ntiles) {
            OddView<Q> v;
            odd_view<Q>(meta + slot1 * kMetaWords, lane, v);
            if (!(v.lk & kSolidBit))
               halves_next = odd_pop_issue<Q>(buf, g, v, lane, pop_s + (stage ^ 1u) * kStageBytes);
         }
         cp_async_commit();
         const uint32_t* m = meta + slot * kMetaWords;
         if (!(m[kMetaLk + lane] & kSolidBit)) {
            const uint32_t* sm = pop + stage * Q * 32;
            float G[Q], o[Q];
#pragma unroll
            for (int s = 0; s < Q; s++) G[s] = word_value<ST>(sm[s * 32 + lane], (halves >> s) & 1u);
            collide_cell<Q, ST, FORCE>(G, o, p);
            OddView<Q> v;
            odd_view<Q>(m, lane, v);
#pragma unroll
            for (int s = 0; s < Q; s++) store_raw(buf + odd_elem<Q>(g, v, s), o[s]);
         }
         if (t1 >= ntiles) break;
         t = t1;
         t1 = t2;
         t2 = t3;
         halves = halves_next;
         slot = slot1;
         stage ^= 1u;
      }
   }
   if (fed) feed_done(p.sched);
}

// Persistent grid: as many blocks as fit on the device at once, queried once
// per device and kernel (the shared-memory opt-in is set at the same time).
template <typename Kern>
cudaError_t persistent_grid(Kern kern, size_t smem, std::atomic<int>* cache, int& grid)
{
   int dev = 0;
   cudaError_t e = cudaGetDevice(&dev);
   if (e != cudaSuccess) return e;
   if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
   int cached = cache[dev].load(std::memory_order_relaxed);
   if (cached == 0) {
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      int per_sm = 0, nsm = 0;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kCompactWarps * 32, smem);
      if (e != cudaSuccess) return e;
      e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      if (per_sm < 1) return cudaErrorInvalidConfiguration;
      cached = per_sm * nsm;
      cache[dev].store(cached, std::memory_order_relaxed);
   }
   grid = cached;
   return cudaSuccess;
}

template <int Q, int ST, bool FORCE>
cudaError_t launch_step_t(int kind, const KParams& p, const CompactGeom& g, void* buf, cudaStream_t stream)
{
   using T = typename Store<ST>::T;
   const size_t smem = kind == K_AA_EVEN ? compact_smem_bytes<Q, ST, K_AA_EVEN>() : compact_smem_bytes<Q, ST, K_AA_ODD>();
   int grid = 0;
   uint32_t ntiles;
   cudaError_t e;
   if (kind == K_AA_EVEN) {
      static std::atomic<int> cache[64];
      e = persistent_grid(compact_even_kernel<Q, ST, FORCE>, smem, cache, grid);
      ntiles = (g.nf + 63) / 64;
   } else {
      static std::atomic<int> cache[64];
      e = persistent_grid(compact_odd_kernel<Q, ST, FORCE>, smem, cache, grid);
      ntiles = g.nrow_tiles;
   }
   if (e != cudaSuccess) return e;
   if (ntiles == 0) return cudaSuccess;
   const uint32_t need = (ntiles + kCompactWarps - 1) / kCompactWarps;
   const unsigned blocks = (unsigned)(need < (uint32_t)grid ? need : (uint32_t)grid);
   T* b = static_cast<T*>(buf);
   if (kind == K_AA_EVEN)
      return launch_overlapped(compact_even_kernel<Q, ST, FORCE>, dim3(blocks), dim3(kCompactWarps * 32), smem, stream,
                               p, g, b);
   return launch_overlapped(compact_odd_kernel<Q, ST, FORCE>, dim3(blocks), dim3(kCompactWarps * 32), smem, stream, p,
                            g, b);
}

template <int Q, int ST>
cudaError_t launch_step_f(int kind, const KParams& p, const CompactGeom& g, void* buf, cudaStream_t stream)
{
   return p.forced ? launch_step_t<Q, ST, true>(kind, p, g, buf, stream)
                   : launch_step_t<Q, ST, false>(kind, p, g, buf, stream);
}

// ------------------------------------------------------------ copies
template <typename T>
__global__ void expand_kernel(const uint32_t* dcell, uint32_t nf, uint32_t cplane, int Q, const T* cbuf, T* dense,
                              int64_t plane)
{
   const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= nf) return;
   const int64_t c = dcell[i];
   for (int s = 0; s < Q; s++) dense[(int64_t)s * plane + c] = cbuf[(uint64_t)s * cplane + i];
}

template <typename T>
__global__ void compress_kernel(const uint32_t* dcell, uint32_t nf, uint32_t cplane, int Q, const T* dense,
                                int64_t plane, T* cbuf)
{
   const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= nf) return;
   const int64_t c = dcell[i];
   for (int s = 0; s < Q; s++) cbuf[(uint64_t)s * cplane + i] = dense[(int64_t)s * plane + c];
}

__global__ void gather_links_kernel(const OddTile* tiles, uint32_t ntiles, const uint32_t* dcell,
                                    const uint32_t* links, int nx, uint32_t* lk)
{
   const uint64_t tl = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
   if (tl >= (uint64_t)ntiles * 32u) return;
   const OddTile& tile = tiles[tl / 32u];
   const uint32_t lane = (uint32_t)(tl % 32u);
   uint32_t w = kSolidBit;
   if (lane < tile.ncell) {
      const uint32_t c = dcell[tile.b[4] + lane];
      const uint32_t x = c % (uint32_t)nx;
      w = (links ? links[c] : 0u) | (x == 0u ? kRowStartBit : 0u) | (x == (uint32_t)nx - 1u ? kRowEndBit : 0u);
   }
   lk[tl] = w;
}

unsigned blocks_of(uint32_t n) { return (n + 255) / 256; }

}  // namespace

cudaError_t launch_compact_step(int Q, int storage, int kind, const KParams& p, const CompactGeom& g, void* buf,
                                cudaStream_t stream)
{
   if (kind != K_AA_EVEN && kind != K_AA_ODD) return cudaErrorInvalidValue;
   if ((uint64_t)Q * (uint64_t)g.cplane >= (1ull << 32) || (g.cplane & 1u)) return cudaErrorInvalidValue;
   if (Q == 19) {
      switch (storage) {
         case ST_F32: return launch_step_f<19, ST_F32>(kind, p, g, buf, stream);
         case ST_BF16: return launch_step_f<19, ST_BF16>(kind, p, g, buf, stream);
         case ST_F16: return launch_step_f<19, ST_F16>(kind, p, g, buf, stream);
         default: return cudaErrorInvalidValue;
      }
   }
   switch (storage) {
      case ST_F32: return launch_step_f<27, ST_F32>(kind, p, g, buf, stream);
      case ST_BF16: return launch_step_f<27, ST_BF16>(kind, p, g, buf, stream);
      case ST_F16: return launch_step_f<27, ST_F16>(kind, p, g, buf, stream);
      default: return cudaErrorInvalidValue;
   }
}

cudaError_t launch_compact_expand(int Q, int storage, const uint32_t* dcell, uint32_t nf, uint32_t cplane,
                                  const void* cbuf, void* dense, int64_t plane, cudaStream_t stream)
{
   if (nf == 0) return cudaSuccess;
   if (storage == ST_F32)
      expand_kernel<uint32_t><<<blocks_of(nf), 256, 0, stream>>>(dcell, nf, cplane, Q, (const uint32_t*)cbuf,
                                                                  (uint32_t*)dense, plane);
   else
      expand_kernel<uint16_t><<<blocks_of(nf), 256, 0, stream>>>(dcell, nf, cplane, Q, (const uint16_t*)cbuf,
                                                                  (uint16_t*)dense, plane);
   return cudaGetLastError();
}

cudaError_t launch_compact_compress(int Q, int storage, const uint32_t* dcell, uint32_t nf, uint32_t cplane,
                                    const void* dense, int64_t plane, void* cbuf, cudaStream_t stream)
{
   if (nf == 0) return cudaSuccess;
   if (storage == ST_F32)
      compress_kernel<uint32_t><<<blocks_of(nf), 256, 0, stream>>>(dcell, nf, cplane, Q, (const uint32_t*)dense,
                                                                    plane, (uint32_t*)cbuf);
   else
      compress_kernel<uint16_t><<<blocks_of(nf), 256, 0, stream>>>(dcell, nf, cplane, Q, (const uint16_t*)dense,
                                                                    plane, (uint16_t*)cbuf);
   return cudaGetLastError();
}

cudaError_t launch_compact_links(const OddTile* tiles, uint32_t ntiles, const uint32_t* dcell,
                                 const uint32_t* links, int nx, uint32_t* lk, cudaStream_t stream)
{
   if (ntiles == 0) return cudaSuccess;
   if (ntiles >= (1u << 27)) return cudaErrorInvalidValue;
   gather_links_kernel<<<blocks_of(ntiles * 32u), 256, 0, stream>>>(tiles, ntiles, dcell, links, nx, lk);
   return cudaGetLastError();
}

}  // namespace lbm
