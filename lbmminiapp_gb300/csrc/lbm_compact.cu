// AA step kernels on the compact fluid-only layout (lbm_compact.cuh) for the
// shifted FP32 / BF16 / FP16 storage with FP32 collision, and the copies
// between the compact and the dense layouts.
//
// Both steps use the pipelined scheme of the dense kernels
// (lbm_step_async_low.cuh): persistent warps, one fluid cell per lane, and the
// populations of the next tile in flight as 4-byte cp.async copies (the
// aligned word holding each element) into a two-stage shared buffer per warp
// while the current tile collides.  No lane holds a solid cell, and every
// sector moved holds fluid populations only.
//
//   even step (KernelAA_SOA_Base.cpp:173-254): tiles of 32 consecutive fluid
//     indices; read own slot opp(s), write own slot s: contiguous accesses.
//   odd step (KernelAA_SOA_Base.cpp:257-342): tiles of up to 32 fluid cells of
//     one row, so the 9 neighbour rows are the same for the whole warp; read
//     slot s at x - c_s (own slot opp(s) when that neighbour is blocked),
//     write slot opp(s) at x + c_s (own slot s when blocked).
//
// AA stays race-free under the prefetch for the dense layout's reason: a
// cell's reads and writes touch the same set of elements, so a prefetch of
// another tile never reads an element this tile writes.  A copied word may
// hold a second element written by another cell; only the lane's own half is
// used.
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

// Shared memory per block: a two-stage buffer per warp of one word per lane
// and direction (the even step's words hold two cells).
template <int Q, int ST, int KIND>
constexpr size_t compact_smem_bytes()
{
   using T = typename Store<ST>::T;
   return (size_t)kCompactWarps * kAsyncStages * Q * 32 *
          (KIND == K_AA_EVEN ? sizeof(typename PairWord<T>::W) : sizeof(uint32_t));
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

// Direction index of the velocity (cx, cy, cz), -1 if the lattice has none.
__host__ __device__ constexpr int dir_of(int Q, int cx, int cy, int cz)
{
   for (int s = 0; s < Q; s++)
      if (lat_c(Q, s, 0) == cx && lat_c(Q, s, 1) == cy && lat_c(Q, s, 2) == cz) return s;
   return -1;
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
   uint32_t t = blockIdx.x * kCompactWarps + warp;
   if (t >= ntiles) return;
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
   issue(t, sbase);
   cp_async_commit();
   int stage = 0;
   for (;;) {
      const uint32_t next = t + nw;
      if (next < ntiles) issue(next, sbase + (stage ^ 1) * kStageBytes);
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
      if (next >= ntiles) break;
      t = next;
      stage ^= 1;
   }
}

// ------------------------------------------------------------------ odd
// Lane state of a row tile.  base[k] is the compact index of (x, row k) as
// if that cell were fluid, rows k = 3 (dy + 1) + (dz + 1); n[k] is the row's
// fluid count, used for the periodic wrap of x at the row ends.
struct OddLane {
   uint32_t i, lk;
   bool active, x0, xl;   // x0: x == 0; xl: x == nx - 1
   uint32_t base[9];
   uint32_t n[9];
};

__device__ __forceinline__ int wrap(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

__device__ __forceinline__ void odd_prepare(const CompactGeom& g, uint32_t row, uint32_t first, int lane,
                                            OddLane& L)
{
   const RowInfo own = g.rows[row];
   L.i = first + (uint32_t)lane;
   L.active = L.i < own.start + own.count;
   const uint32_t ii = L.active ? L.i : first;
   const int x = (int)__ldg(g.xs + ii);
   L.lk = __ldg(g.lk + ii);
   L.x0 = x == 0;
   L.xl = x == g.nx - 1;
   const uint32_t z = div_magic(row, (uint32_t)g.ny, g.m_ny);
   const int y = (int)(row - z * (uint32_t)g.ny);
#pragma unroll
   for (int k = 0; k < 9; k++) {
      if (k == 4) {
         L.base[4] = L.i;
         L.n[4] = own.count;
         continue;
      }
      const int dy = k / 3 - 1, dz = k % 3 - 1;
      const uint32_t r2 = (uint32_t)wrap(y + dy, g.ny) + (uint32_t)g.ny * (uint32_t)wrap((int)z + dz, g.nz);
      const RowInfo ri = g.rows[r2];
      L.base[k] = ri.start + (uint32_t)__ldg(g.pre + (r2 * (uint32_t)g.nx + (uint32_t)x));
      L.n[k] = ri.count;
   }
}

// Compact index of the fluid neighbour at x + (dx, dy, dz).
template <int Q>
__device__ __forceinline__ uint32_t nbr_index(const OddLane& L, int dx, int dy, int dz)
{
   const int k = (dy + 1) * 3 + (dz + 1);
   if (dx == 0) return L.base[k];
   if (dx < 0) return L.base[k] - 1u + (L.x0 ? L.n[k] : 0u);
   // x + 1: one past (x, row k) when that cell is fluid
   const uint32_t fl = k == 4 ? 1u : (((L.lk >> dir_of(Q, 0, dy, dz)) & 1u) ^ 1u);
   return L.base[k] + fl - (L.xl ? L.n[k] : 0u);
}

template <int Q, typename T>
__device__ __forceinline__ uint32_t odd_issue(const T* buf, const CompactGeom& g, const OddLane& L, int lane,
                                              uint32_t sb)
{
   uint32_t halves = 0u;
   if (!L.active) return halves;
#pragma unroll
   for (int s = 0; s < Q; s++) {
      const int o = lat_opp(Q, s);
      uint32_t e;
      if (s == lat_rest(Q) || ((L.lk >> o) & 1u)) e = g.soff[s == lat_rest(Q) ? s : o] + L.i;
      else e = g.soff[s] + nbr_index<Q>(L, -lat_c(Q, s, 0), -lat_c(Q, s, 1), -lat_c(Q, s, 2));
      cp_async4(sb + (uint32_t)(s * 32 + lane) * 4u, word_of(buf, e));
      if constexpr (sizeof(T) == 2) halves |= (e & 1u) << s;
   }
   return halves;
}

template <int Q, int ST, bool FORCE>
__global__ void __launch_bounds__(kCompactWarps * 32, 2) compact_odd_kernel(const KParams p, const CompactGeom g,
                                                                            typename Store<ST>::T* buf)
{
   extern __shared__ __align__(16) uint32_t compact_smem[];
   const int lane = threadIdx.x & 31;
   const int warp = threadIdx.x >> 5;
   const uint32_t ntiles = g.nrow_tiles;
   const uint32_t nw = gridDim.x * kCompactWarps;
   uint32_t t = blockIdx.x * kCompactWarps + warp;
   if (t >= ntiles) return;
   wait_prior_grid();
   uint32_t* mine = compact_smem + (size_t)warp * kAsyncStages * Q * 32;
   const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(mine);
   constexpr uint32_t kStageBytes = Q * 32 * 4;
   OddLane cur;
   odd_prepare(g, __ldg(g.tile_row + t), __ldg(g.tile_first + t), lane, cur);
   uint32_t halves = odd_issue<Q>(buf, g, cur, lane, sbase);
   cp_async_commit();
   // the tile table one tile ahead of the prefetch
   uint32_t row_ahead = 0u, first_ahead = 0u;
   if (t + nw < ntiles) {
      row_ahead = __ldg(g.tile_row + t + nw);
      first_ahead = __ldg(g.tile_first + t + nw);
   }
   int stage = 0;
   for (;;) {
      const uint32_t next = t + nw;
      OddLane nxt = cur;
      uint32_t halves_next = 0u;
      if (next < ntiles) {
         odd_prepare(g, row_ahead, first_ahead, lane, nxt);
         if (next + nw < ntiles) {
            row_ahead = __ldg(g.tile_row + next + nw);
            first_ahead = __ldg(g.tile_first + next + nw);
         }
         halves_next = odd_issue<Q>(buf, g, nxt, lane, sbase + (stage ^ 1) * kStageBytes);
      }
      cp_async_commit();
      cp_async_wait_prev();
      if (cur.active) {
         const uint32_t* sm = mine + stage * Q * 32;
         float G[Q], o[Q];
#pragma unroll
         for (int s = 0; s < Q; s++) G[s] = word_value<ST>(sm[s * 32 + lane], (halves >> s) & 1u);
         collide_cell<Q, ST, FORCE>(G, o, p);
#pragma unroll
         for (int s = 0; s < Q; s++) {
            uint32_t e;
            if (s == lat_rest(Q) || ((cur.lk >> s) & 1u)) e = g.soff[s] + cur.i;
            else e = g.soff[lat_opp(Q, s)] + nbr_index<Q>(cur, lat_c(Q, s, 0), lat_c(Q, s, 1), lat_c(Q, s, 2));
            store_raw(buf + e, o[s]);
         }
      }
      if (next >= ntiles) break;
      t = next;
      cur = nxt;
      halves = halves_next;
      stage ^= 1;
   }
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

__global__ void gather_links_kernel(const uint32_t* dcell, const uint32_t* links, uint32_t* lk, uint32_t nf)
{
   const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i < nf) lk[i] = links ? links[dcell[i]] : 0u;
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

cudaError_t launch_compact_links(const uint32_t* dcell, const uint32_t* links, uint32_t* lk, uint32_t nf,
                                 cudaStream_t stream)
{
   if (nf == 0) return cudaSuccess;
   gather_links_kernel<<<blocks_of(nf), 256, 0, stream>>>(dcell, links, lk, nf);
   return cudaGetLastError();
}

}  // namespace lbm
