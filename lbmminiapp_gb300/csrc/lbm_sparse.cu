// Compact fluid-only layout: the reference's own population buffers and
// adjacency list.
//
// The reference stores populations only for fluid points, direction s of
// fluid point i at dstrb[nFluid*s + i], and streams through an int32
// adjacency list built by GeometryAAAB::setupAdjacency
// (src/geometries/GeometryAAAB.cpp:18-124): adjacency[nFluid*s + i] is the
// element index of slot s at the neighbour x - c_s (AA, AB pull) or x + c_s
// (AB push), or of the own slot opp(s) when that neighbour is a wall.  These
// kernels run the same steps on those buffers, so a caller that already
// holds the reference's geometry can keep its layout and ordering:
//
//   AA even  (KernelAA_SOA_Base.cpp:173-254): d_s = dstrb[nF*opp(s) + i], out_s -> dstrb[nF*s + i]
//   AA odd   (KernelAA_SOA_Base.cpp:257-342): loc_s = adj[nF*s + i], d_s = dstrb[loc_s],
//            out_s -> dstrb[loc_opp(s)]
//   AB push  (KernelAB_SOA_Base.cpp:111-186): d_s = src[nF*s + i], out_s -> tgt[adj[nF*s + i]]
//   AB pull  (KernelAB_SOA_Pull.cpp:113-194): d_s = src[adj[nF*s + i]], out_s -> tgt[nF*s + i]
//
// One thread per fluid index; FP64 storage with the exact reference-order
// arithmetic or F64X.  The layout suits media with few fluid cells, where
// a dense grid would hold and scan every solid cell; the price is the
// 4*Q bytes of adjacency each AA odd / AB update reads.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/lbm_gb300.h"
#include "lbm_f64x.cuh"
#include "lbm_launch.cuh"
#include "lbm_step_async.cuh"

using namespace lbm;

struct lbm_sparse_handle {
   int Q = 19;
   int pattern = LBM_PATTERN_AA;
   int pull = 0;
   int arith = AR_F64X;
   int device = 0;
   int64_t nfluid = 0;
   int32_t* adj = nullptr;   // device [Q][nfluid]
   KParams params;
   cudaStream_t stream = nullptr;
   std::string err;
};

namespace {

constexpr int kSparseThreads = 256;

lbm_status sfail(lbm_sparse_handle* h, lbm_status s, const char* fmt, ...)
{
   if (h) {
      char buf[512];
      va_list ap;
      va_start(ap, fmt);
      vsnprintf(buf, sizeof(buf), fmt, ap);
      va_end(ap);
      h->err = buf;
   }
   return s;
}

// D3Q19: two blocks per SM (at most 128 registers; the AA even step alone
// wanted 140, which left one block per SM and made it slower than the odd
// step).
template <int Q>
constexpr int sparse_min_blocks() { return Q == 19 ? 2 : 1; }

template <int Q, int AR, int KIND>
__global__ void __launch_bounds__(kSparseThreads, sparse_min_blocks<Q>()) sparse_step_kernel(const KParams p, const int32_t* __restrict__ adj,
                                                                     int64_t nfluid, int64_t start, int64_t count,
                                                                     const double* src, double* dst)
{
   const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
   wait_prior_grid();
   if (k >= count) return;
   const int64_t i = start + k;
   // Element indices fit 32 bits: the reference's int32 adjacency requires
   // Q * nFluid < 2^31.
   const uint32_t nf = (uint32_t)nfluid, ii = (uint32_t)i;
   uint32_t loc[Q];
   double d[Q];
#pragma unroll
   for (int s = 0; s < Q; s++) {
      if (KIND == K_AA_EVEN) loc[s] = nf * (uint32_t)lat_opp(Q, s) + ii;
      else if (KIND == K_AB_PUSH) loc[s] = nf * (uint32_t)s + ii;
      else loc[s] = (uint32_t)adj[(size_t)nf * s + ii];
      d[s] = src[loc[s]];
   }
   double o[Q];
   if constexpr (AR == AR_F64) {
      collide_f64<Q>(d, o, p.F[0], p.F[1], p.F[2], 0.0, p);
   } else {
      uint64_t bits[Q];
#pragma unroll
      for (int s = 0; s < Q; s++) bits[s] = x64::double_bits(d[s]);
      collide_f64x<Q>(bits, p);
#pragma unroll
      for (int s = 0; s < Q; s++) o[s] = x64::as_double(bits[s]);
   }
#pragma unroll
   for (int s = 0; s < Q; s++) {
      uint32_t w;
      if (KIND == K_AA_EVEN || KIND == K_AB_PULL) w = nf * (uint32_t)s + ii;
      else if (KIND == K_AA_ODD) w = loc[lat_opp(Q, s)];
      else w = (uint32_t)adj[(size_t)nf * s + ii];
      dst[w] = o[s];
   }
}

// Pipelined form for F64X: persistent warps on tiles of 32 consecutive fluid
// indices, the next tile's populations prefetched with 8-byte cp.async into a
// two-stage shared buffer per warp while the current tile collides (the
// dense grid's scheme, lbm_step_async.cuh).  The gather kinds (AA odd, AB
// pull) need the next tile's adjacency to issue those copies, so each lane
// loads it one tile further ahead into registers; the scatter kinds (AA odd,
// AB push) load the current tile's write locations when its collision starts,
// and each output is stored as the collision makes it.  AA stays race-free
// under the prefetch: a fluid point's read and write locations are the same
// set, disjoint from every other point's.
constexpr int kSparseAsyncWarps = 4;
constexpr int kSparseAsyncBlocks = 3;

template <int KIND>
constexpr bool sparse_gathers() { return KIND == K_AA_ODD || KIND == K_AB_PULL; }
template <int KIND>
constexpr bool sparse_scatters() { return KIND == K_AA_ODD || KIND == K_AB_PUSH; }

template <int Q, int KIND>
struct SparseEmit {
   double* dst;
   uint32_t nf, i;
   const uint32_t (&wl)[Q];   // write locations (scatter kinds)
   __device__ __forceinline__ void operator()(int s, uint64_t v) const
   {
      const uint32_t w = sparse_scatters<KIND>() ? wl[s] : nf * (uint32_t)s + i;
      reinterpret_cast<unsigned long long*>(dst)[w] = v;
   }
};

template <int Q, int KIND>
__global__ void __launch_bounds__(kSparseAsyncWarps * 32, kSparseAsyncBlocks) sparse_async_kernel(
   const KParams p, const int32_t* __restrict__ adj, uint32_t nf, uint32_t start, uint32_t count, uint32_t ntiles,
   const double* src, double* dst)
{
   extern __shared__ __align__(16) unsigned long long sparse_smem[];
   const int lane = threadIdx.x & 31;
   const int warp = threadIdx.x >> 5;
   const uint32_t nw = gridDim.x * kSparseAsyncWarps;
   wait_prior_grid();
   unsigned long long* mine = sparse_smem + (size_t)warp * kAsyncStages * Q * 32;
   const uint32_t sbase = (uint32_t)__cvta_generic_to_shared(mine);
   constexpr uint32_t kStageBytes = Q * 32 * 8;
   const unsigned long long* s64 = reinterpret_cast<const unsigned long long*>(src);
   // fluid index of this lane in tile tt, and whether it is inside the range
   auto point = [&](uint32_t tt, bool& act) {
      const uint32_t k = tt * 32u + (uint32_t)lane;
      act = k < count;
      return start + k;
   };
   uint32_t ahead[Q];   // read locations of the tile to be issued next (gather kinds)
   auto load_ahead = [&](uint32_t tt) {
      bool act;
      const uint32_t i = point(tt, act);
#pragma unroll
      for (int s = 0; s < Q; s++) ahead[s] = act ? (uint32_t)__ldg(adj + (size_t)nf * s + i) : 0u;
   };
   auto issue = [&](uint32_t tt, uint32_t sb) {
      bool act;
      const uint32_t i = point(tt, act);
      if (!act) return;
#pragma unroll
      for (int s = 0; s < Q; s++) {
         uint32_t r;
         if (KIND == K_AA_EVEN) r = nf * (uint32_t)lat_opp(Q, s) + i;
         else if (KIND == K_AB_PUSH) r = nf * (uint32_t)s + i;
         else r = ahead[s];
         cp_async8(sb + (uint32_t)(s * 32 + lane) * 8u, s64 + r);
      }
   };
   // tiles: three per warp in a fixed order, then the launch's tile feed (8
   // counters for the D3Q19 tiles, which it hands out fastest); t is collided
   // while t1's populations are in flight and t2's read locations are loaded
   const bool fed = feed_on(ntiles, nw);
   TileFeed feed{0u, 0u, 1u, false};
   if (fed)
      feed = feed_start(p.sched, 3u * nw, ntiles, blockIdx.x * kSparseAsyncWarps + warp, nw,
                        Q == 19 ? kFeedGroups : 1u, lane);
   uint32_t t = blockIdx.x * kSparseAsyncWarps + warp;
   if (t < ntiles) {
      uint32_t t1 = t + nw < ntiles ? t + nw : ntiles;
      uint32_t t2 = t + 2u * nw < ntiles ? t + 2u * nw : ntiles;
      if (sparse_gathers<KIND>()) load_ahead(t);
      issue(t, sbase);
      cp_async_commit();
      if (sparse_gathers<KIND>() && t1 < ntiles) load_ahead(t1);
      int stage = 0;
      for (;;) {
         if (t1 < ntiles) {
            issue(t1, sbase + (stage ^ 1) * kStageBytes);
            if (sparse_gathers<KIND>() && t2 < ntiles) load_ahead(t2);
         }
         cp_async_commit();
         cp_async_wait_prev();
         bool act;
         const uint32_t i = point(t, act);
         if (act) {
            uint32_t wl[Q];
            if (sparse_scatters<KIND>()) {
#pragma unroll
               for (int s = 0; s < Q; s++) {
                  const int r = KIND == K_AA_ODD ? lat_opp(Q, s) : s;
                  wl[s] = (uint32_t)__ldg(adj + (size_t)nf * r + i);
               }
            }
            const SparseEmit<Q, KIND> emit{dst, nf, i, wl};
            collide_f64x_shared_emit<Q>(mine + stage * Q * 32 + lane, p, emit);
         }
         if (t1 >= ntiles) break;
         t = t1;
         t1 = t2;
         t2 = feed_after(feed, fed, t2, p.sched, 3u * nw, ntiles, nw, lane);
         stage ^= 1;
      }
   }
   if (fed) feed_done(p.sched);
}

template <int Q, int KIND>
cudaError_t launch_sparse_async(const KParams& p, const int32_t* adj, int64_t nfluid, int64_t start, int64_t count,
                                const double* src, double* dst, cudaStream_t stream)
{
   // persistent grid per device ordinal, set once (any thread computes the same value)
   static std::atomic<int> grid_of_device[64];
   int dev = 0;
   cudaError_t e = cudaGetDevice(&dev);
   if (e != cudaSuccess) return e;
   if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
   auto kern = sparse_async_kernel<Q, KIND>;
   constexpr size_t smem = (size_t)kSparseAsyncWarps * kAsyncStages * Q * 32 * sizeof(unsigned long long);
   int cached = grid_of_device[dev].load(std::memory_order_relaxed);
   if (cached == 0) {
      e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      if (e != cudaSuccess) return e;
      int per_sm = 0, nsm = 0;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kSparseAsyncWarps * 32, smem);
      if (e != cudaSuccess) return e;
      e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
      if (e != cudaSuccess) return e;
      if (per_sm < 1) return cudaErrorInvalidConfiguration;
      cached = per_sm * nsm;
      grid_of_device[dev].store(cached, std::memory_order_relaxed);
   }
   const uint32_t ntiles = (uint32_t)((count + 31) / 32);
   const uint32_t need = (ntiles + kSparseAsyncWarps - 1) / kSparseAsyncWarps;
   const unsigned grid = (unsigned)(need < (uint32_t)cached ? need : (uint32_t)cached);
   return launch_overlapped(kern, dim3(grid), dim3(kSparseAsyncWarps * 32), smem, stream, p, adj, (uint32_t)nfluid,
                            (uint32_t)start, (uint32_t)count, ntiles, src, dst);
}

template <int Q, int AR>
cudaError_t launch_sparse_q(int kind, const KParams& p, const int32_t* adj, int64_t nfluid, int64_t start,
                            int64_t count, const double* src, double* dst, cudaStream_t stream)
{
   if (AR == AR_F64X) {
      switch (kind) {
         case K_AA_EVEN: return launch_sparse_async<Q, K_AA_EVEN>(p, adj, nfluid, start, count, src, dst, stream);
         case K_AA_ODD: return launch_sparse_async<Q, K_AA_ODD>(p, adj, nfluid, start, count, src, dst, stream);
         case K_AB_PUSH: return launch_sparse_async<Q, K_AB_PUSH>(p, adj, nfluid, start, count, src, dst, stream);
         default: return launch_sparse_async<Q, K_AB_PULL>(p, adj, nfluid, start, count, src, dst, stream);
      }
   }
   const dim3 grid((unsigned)((count + kSparseThreads - 1) / kSparseThreads)), block(kSparseThreads);
   switch (kind) {
      case K_AA_EVEN:
         return launch_overlapped(sparse_step_kernel<Q, AR, K_AA_EVEN>, grid, block, 0, stream, p, adj, nfluid, start,
                                  count, src, dst);
      case K_AA_ODD:
         return launch_overlapped(sparse_step_kernel<Q, AR, K_AA_ODD>, grid, block, 0, stream, p, adj, nfluid, start,
                                  count, src, dst);
      case K_AB_PUSH:
         return launch_overlapped(sparse_step_kernel<Q, AR, K_AB_PUSH>, grid, block, 0, stream, p, adj, nfluid, start,
                                  count, src, dst);
      default:
         return launch_overlapped(sparse_step_kernel<Q, AR, K_AB_PULL>, grid, block, 0, stream, p, adj, nfluid, start,
                                  count, src, dst);
   }
}

lbm_status sparse_launch(lbm_sparse_handle* h, int kind, const void* src, void* dst, int64_t start, int64_t count)
{
   if (!h) return LBM_ERR_INVALID_ARGUMENT;
   if (!src || !dst) return sfail(h, LBM_ERR_INVALID_ARGUMENT, "null population buffer");
   if (start < 0 || count < 0 || start + count > h->nfluid)
      return sfail(h, LBM_ERR_INVALID_ARGUMENT, "range [%lld, %lld) outside [0, %lld)", (long long)start,
                   (long long)(start + count), (long long)h->nfluid);
   if (count == 0) return LBM_OK;
   int cur = -1;
   if (cudaGetDevice(&cur) != cudaSuccess || cur != h->device) {
      cudaError_t e = cudaSetDevice(h->device);
      if (e != cudaSuccess) return sfail(h, LBM_ERR_CUDA, "cudaSetDevice: %s", cudaGetErrorString(e));
   }
   const double* s = static_cast<const double*>(src);
   double* d = static_cast<double*>(dst);
   cudaError_t e;
   if (h->Q == 19)
      e = h->arith == AR_F64 ? launch_sparse_q<19, AR_F64>(kind, h->params, h->adj, h->nfluid, start, count, s, d, h->stream)
                             : launch_sparse_q<19, AR_F64X>(kind, h->params, h->adj, h->nfluid, start, count, s, d, h->stream);
   else
      e = h->arith == AR_F64 ? launch_sparse_q<27, AR_F64>(kind, h->params, h->adj, h->nfluid, start, count, s, d, h->stream)
                             : launch_sparse_q<27, AR_F64X>(kind, h->params, h->adj, h->nfluid, start, count, s, d, h->stream);
   if (e != cudaSuccess) return sfail(h, LBM_ERR_CUDA, "sparse step launch: %s", cudaGetErrorString(e));
   return LBM_OK;
}

}  // namespace

extern "C" {

lbm_status lbm_sparse_create(const lbm_config* cfg, int64_t nfluid, const int32_t* adjacency, lbm_sparse_handle** out)
{
   if (!out) return LBM_ERR_INVALID_ARGUMENT;
   *out = nullptr;
   if (!cfg || !adjacency) return LBM_ERR_INVALID_ARGUMENT;
   if (cfg->lattice != 19 && cfg->lattice != 27) return LBM_ERR_INVALID_ARGUMENT;
   if (cfg->prop_pattern != LBM_PATTERN_AA && cfg->prop_pattern != LBM_PATTERN_AB) return LBM_ERR_INVALID_ARGUMENT;
   if (cfg->storage != LBM_STORE_F64) return LBM_ERR_UNSUPPORTED;
   if (cfg->arithmetic != LBM_ARITH_AUTO && cfg->arithmetic != LBM_ARITH_F64 && cfg->arithmetic != LBM_ARITH_F64X)
      return LBM_ERR_UNSUPPORTED;
   const int Q = cfg->lattice;
   // The reference's int32 slot indices limit Q * nFluid to 2^31 - 1.
   if (nfluid <= 0 || (int64_t)Q * nfluid > 0x7FFFFFFFll) return LBM_ERR_INVALID_ARGUMENT;
   const int64_t n = (int64_t)Q * nfluid;
   for (int64_t k = 0; k < n; k++)
      if (adjacency[k] < 0 || (int64_t)adjacency[k] >= n) return LBM_ERR_INVALID_ARGUMENT;
   lbm_sparse_handle* h = new (std::nothrow) lbm_sparse_handle();
   if (!h) return LBM_ERR_OUT_OF_MEMORY;
   h->Q = Q;
   h->pattern = cfg->prop_pattern;
   h->pull = cfg->pull ? 1 : 0;
   h->arith = cfg->arithmetic == LBM_ARITH_F64 ? AR_F64 : AR_F64X;
   h->device = cfg->device;
   h->nfluid = nfluid;
   std::memset(&h->params, 0, sizeof(h->params));
   set_collision_constants(h->params, Q, cfg->omega, cfg->force,
                           (cfg->unroll && Q == 19 && cfg->prop_pattern == LBM_PATTERN_AA) ? 1 : 0);
   cudaError_t e = cudaSetDevice(cfg->device);
   const size_t bytes = (size_t)n * sizeof(int32_t);
   if (e == cudaSuccess && cfg->max_device_bytes && bytes > cfg->max_device_bytes) {
      delete h;
      return LBM_ERR_OUT_OF_MEMORY;
   }
   // the adjacency, then the tile counters of the persistent kernels (zero)
   const size_t sched_off = (bytes + 127) / 128 * 128;
   if (e == cudaSuccess) e = cudaMalloc(&h->adj, sched_off + 4 * kFeedWords);
   if (e == cudaSuccess) e = cudaMemcpy(h->adj, adjacency, bytes, cudaMemcpyHostToDevice);
   if (e == cudaSuccess) e = cudaMemset(reinterpret_cast<char*>(h->adj) + sched_off, 0, 4 * kFeedWords);
   if (e == cudaSuccess) h->params.sched = reinterpret_cast<uint32_t*>(reinterpret_cast<char*>(h->adj) + sched_off);
   if (e != cudaSuccess) {
      cudaGetLastError();
      if (h->adj) cudaFree(h->adj);
      const bool oom = e == cudaErrorMemoryAllocation;
      delete h;
      return oom ? LBM_ERR_OUT_OF_MEMORY : LBM_ERR_CUDA;
   }
   *out = h;
   return LBM_OK;
}

void lbm_sparse_destroy(lbm_sparse_handle* h)
{
   if (!h) return;
   if (h->adj) {
      cudaSetDevice(h->device);
      cudaFree(h->adj);
   }
   delete h;
}

const char* lbm_sparse_last_error(const lbm_sparse_handle* h)
{
   if (!h) return "null handle";
   return h->err.c_str();
}

lbm_status lbm_sparse_set_stream(lbm_sparse_handle* h, void* stream)
{
   if (!h) return LBM_ERR_INVALID_ARGUMENT;
   h->stream = static_cast<cudaStream_t>(stream);
   return LBM_OK;
}

lbm_status lbm_sparse_timestep_even_force(lbm_sparse_handle* h, double* dstrb, int64_t start, int64_t count)
{
   if (!h) return LBM_ERR_INVALID_ARGUMENT;
   if (h->pattern != LBM_PATTERN_AA) return sfail(h, LBM_ERR_STATE, "even/odd steps need an AA handle");
   return sparse_launch(h, K_AA_EVEN, dstrb, dstrb, start, count);
}

lbm_status lbm_sparse_timestep_odd_force(lbm_sparse_handle* h, double* dstrb, int64_t start, int64_t count)
{
   if (!h) return LBM_ERR_INVALID_ARGUMENT;
   if (h->pattern != LBM_PATTERN_AA) return sfail(h, LBM_ERR_STATE, "even/odd steps need an AA handle");
   return sparse_launch(h, K_AA_ODD, dstrb, dstrb, start, count);
}

lbm_status lbm_sparse_timestep_force(lbm_sparse_handle* h, const double* src, double* tgt, int64_t start,
                                     int64_t count)
{
   if (!h) return LBM_ERR_INVALID_ARGUMENT;
   if (h->pattern != LBM_PATTERN_AB) return sfail(h, LBM_ERR_STATE, "timestep_force needs an AB handle");
   if (src == tgt) return sfail(h, LBM_ERR_INVALID_ARGUMENT, "AB needs two distinct buffers");
   return sparse_launch(h, h->pull ? K_AB_PULL : K_AB_PUSH, src, tgt, start, count);
}

}  // extern "C"
