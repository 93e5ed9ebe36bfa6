// Auxiliary device kernels: link words, initialisation, population import /
// export, macroscopic readouts and the FP64 conservation reduction.  None of
// these is on the per-step hot path.
#pragma once

#include <cuda_runtime.h>

#include "lbm_physics.cuh"

namespace lbm {

struct GridDims {
   int nx, ny, nz;
   int64_t ncell, plane;
   int periodic[3];
};

__device__ __forceinline__ bool cell_xyz(const GridDims& g, int64_t c, int& x, int& y, int& z)
{
   if (c >= g.ncell) return false;
   if (c < (int64_t)0xFFFFFFFF) {
      // 32-bit divisions (a 64-bit one is a long software sequence)
      const uint32_t c32 = (uint32_t)c, r = c32 / (uint32_t)g.nx;
      x = (int)(c32 - r * (uint32_t)g.nx);
      const uint32_t q = r / (uint32_t)g.ny;
      y = (int)(r - q * (uint32_t)g.ny);
      z = (int)q;
      return true;
   }
   x = (int)(c % g.nx);
   const int64_t r = c / g.nx;
   y = (int)(r % g.ny);
   z = (int)(r / g.ny);
   return true;
}

// Neighbour of (x,y,z) along (sx,sy,sz); returns -1 when it leaves the box
// through a non-periodic face.
__device__ __forceinline__ int64_t nbr_cell(const GridDims& g, int x, int y, int z, int sx, int sy, int sz)
{
   int p[3] = {x + sx, y + sy, z + sz};
   const int n[3] = {g.nx, g.ny, g.nz};
#pragma unroll
   for (int d = 0; d < 3; d++) {
      if (p[d] < 0 || p[d] >= n[d]) {
         if (!g.periodic[d]) return -1;
         p[d] = p[d] < 0 ? p[d] + n[d] : p[d] - n[d];
      }
   }
   return (int64_t)p[0] + (int64_t)g.nx * ((int64_t)p[1] + (int64_t)g.ny * p[2]);
}

template <int Q>
__global__ void build_links_kernel(GridDims g, const uint8_t* solid, uint32_t* links)
{
   const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
   int x, y, z;
   if (!cell_xyz(g, c, x, y, z)) return;
   if (solid && solid[c]) {
      links[c] = kSolidBit;
      return;
   }
   uint32_t w = 0;
#pragma unroll
   for (int s = 0; s < Q; s++) {
      if (s == lat_rest(Q)) continue;
      const int64_t n = nbr_cell(g, x, y, z, lat_c(Q, s, 0), lat_c(Q, s, 1), lat_c(Q, s, 2));
      if (n < 0 || (solid && solid[n])) w |= 1u << s;
   }
   links[c] = w;
}

// Stored value <-> population f.
template <int ST>
__device__ __forceinline__ double load_pop(const void* buf, int64_t idx, double w)
{
   if constexpr (ST == ST_F64) {
      return static_cast<const double*>(buf)[idx];
   } else {
      const float g = load_shifted(static_cast<const typename Store<ST>::T*>(buf) + idx);
      return (double)g + w;
   }
}

template <int ST>
__device__ __forceinline__ void store_pop(void* buf, int64_t idx, double f, double w)
{
   if constexpr (ST == ST_F64) {
      static_cast<double*>(buf)[idx] = f;
   } else {
      store_shifted(static_cast<typename Store<ST>::T*>(buf) + idx, (float)(f - w));
   }
}

// Signed sum c_0 a_0 + c_1 a_1 + c_2 a_2 for the compile-time direction S,
// with the zero terms left out and c = +-1 as an add or subtract: the same
// value as the reference's c . a (adding +-0 to a sum, or multiplying by
// +-1, is exact).
template <int Q, int S>
__device__ __forceinline__ double cdot_d(double a0, double a1, double a2)
{
   constexpr int c0 = lat_c(Q, S, 0), c1 = lat_c(Q, S, 1), c2 = lat_c(Q, S, 2);
   double r = 0.0;
   if (c0 != 0) r = c0 > 0 ? a0 : -a0;
   if (c1 != 0) r = c0 != 0 ? (c1 > 0 ? r + a1 : r - a1) : (c1 > 0 ? a1 : -a1);
   if (c2 != 0) r = (c0 != 0 || c1 != 0) ? (c2 > 0 ? r + a2 : r - a2) : (c2 > 0 ? a2 : -a2);
   return r;
}

template <int Q, int ST, int S = 0>
__device__ __forceinline__ void init_eq_dirs(const GridDims& g, int64_t c, double r, double u0, double u1,
                                             double u2, double huu, void* b0, void* b1, int aa)
{
   if constexpr (S < Q) {
      const double cu = 3.0 * cdot_d<Q, S>(u0, u1, u2);
      constexpr double w = lat_w(Q, S);
      const double f = w * r * (1.0 + cu + 0.5 * cu * cu - huu);
      if (aa) {
         constexpr int o = lat_opp(Q, S);
         store_pop<ST>(b0, (int64_t)o * g.plane + c, f, lat_w(Q, o));
      } else {
         store_pop<ST>(b0, (int64_t)S * g.plane + c, f, w);
         store_pop<ST>(b1, (int64_t)S * g.plane + c, f, w);
      }
      init_eq_dirs<Q, ST, S + 1>(g, c, r, u0, u1, u2, huu, b0, b1, aa);
   }
}

// Reference equilibrium w rho (1 + cu + cu^2/2 - uu/2)
// (src/kernels/KernelAA_SOA_Base.cpp:229-236) for the cells [c0, c0+count);
// rho[k] and u[d*in_stride + k] hold cell c0+k, and default to 1 / 0.
template <int Q, int ST>
__global__ void init_eq_kernel(GridDims g, int64_t c0, int64_t count, const double* rho, const double* u,
                               int64_t in_stride, void* b0, void* b1, int aa)
{
   const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
   if (k >= count) return;
   const int64_t c = c0 + k;
   const double r = rho ? rho[k] : 1.0;
   const double u0 = u ? u[k] : 0.0, u1 = u ? u[in_stride + k] : 0.0, u2 = u ? u[2 * in_stride + k] : 0.0;
   const double uu = 3.0 * (u0 * u0 + u1 * u1 + u2 * u2);
   init_eq_dirs<Q, ST>(g, c, r, u0, u1, u2, 0.5 * uu, b0, b1, aa);
}

// Weight and velocity component of a direction known only at run time,
// selected from compile-time constants (indexing the constexpr tables with a
// run-time index would copy them to local memory).
template <int Q>
__device__ __forceinline__ double weight_at(int r)
{
   double w = 0.0;
#pragma unroll
   for (int s = 0; s < Q; s++)
      if (s == r) w = lat_w(Q, s);
   return w;
}
template <int Q>
__device__ __forceinline__ int velocity_at(int r, int d)
{
   int v = 0;
#pragma unroll
   for (int s = 0; s < Q; s++)
      if (s == r) v = d == 0 ? lat_c(Q, s, 0) : (d == 1 ? lat_c(Q, s, 1) : lat_c(Q, s, 2));
   return v;
}

// One direction plane from a dense double plane into slot `slot` of up to two
// buffers.
template <int ST>
__global__ void import_plane_kernel(GridDims g, const double* src, int slot, double w, void* b0, void* b1)
{
   const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
   if (c >= g.ncell) return;
   const double f = src[c];
   store_pop<ST>(b0, (int64_t)slot * g.plane + c, f, w);
   if (b1) store_pop<ST>(b1, (int64_t)slot * g.plane + c, f, w);
}

// Export direction s as a dense double plane.  mode 0: raw slot s; mode 1:
// own slot opp(s) (AA at even time); mode 2: pull gather (slot s at x - c_s,
// or own slot opp(s) when that neighbour is blocked).  NaN at solid cells.
// Direction s of a plane kernel with its constants, made on the host.
struct PlaneDir {
   int s, o, rest;
   int c[3];
   double w_s, w_o;
};

inline PlaneDir plane_dir(int Q, int s)
{
   PlaneDir d;
   d.s = s;
   d.o = lat_opp(Q, s);
   d.rest = s == lat_rest(Q);
   for (int k = 0; k < 3; k++) d.c[k] = lat_c(Q, s, k);
   d.w_s = lat_w(Q, s);
   d.w_o = lat_w(Q, d.o);
   return d;
}

template <int Q, int ST>
__global__ void export_plane_kernel(GridDims g, const void* buf, const uint32_t* links, PlaneDir pd, int mode,
                                    double* dst)
{
   const int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
   int x, y, z;
   if (!cell_xyz(g, c, x, y, z)) return;
   const uint32_t lk = links ? links[c] : 0u;
   if (lk & kSolidBit) {
      dst[c] = __longlong_as_double(0x7FF8000000000000LL);
      return;
   }
   int64_t idx;
   double w;
   if (mode == 0) {
      w = pd.w_s;
      idx = (int64_t)pd.s * g.plane + c;
   } else if (mode == 1 || pd.rest || ((lk >> pd.o) & 1u)) {
      w = pd.w_o;
      idx = (int64_t)pd.o * g.plane + c;
   } else {
      w = pd.w_s;
      const int64_t n = nbr_cell(g, x, y, z, -pd.c[0], -pd.c[1], -pd.c[2]);
      idx = (int64_t)pd.s * g.plane + n;
   }
   dst[c] = load_pop<ST>(buf, idx, w);
}

// Logical population of direction s at cell c (same modes as export).
template <int Q, int ST>
__device__ __forceinline__ double logical_pop(const GridDims& g, const void* buf, uint32_t lk, int x, int y,
                                              int z, int64_t c, int s, int mode)
{
   const int o = lat_opp(Q, s);
   if (mode == 0) return load_pop<ST>(buf, (int64_t)s * g.plane + c, lat_w(Q, s));
   if (mode == 1 || s == lat_rest(Q) || ((lk >> o) & 1u))
      return load_pop<ST>(buf, (int64_t)o * g.plane + c, lat_w(Q, o));
   const int64_t n = nbr_cell(g, x, y, z, -lat_c(Q, s, 0), -lat_c(Q, s, 1), -lat_c(Q, s, 2));
   return load_pop<ST>(buf, (int64_t)s * g.plane + n, lat_w(Q, s));
}

// rho and u = sum(c f)/rho (no F/2 shift) for the cells [c0, c0+count);
// cell c0+k goes to rho[k] and u[d*out_stride + k]; NaN at solid cells.
// Zero stencil terms are left out and +-1 terms become adds or subtracts,
// which gives the same sums as the reference's f * c accumulation.
template <int Q, int ST>
__global__ void macros_kernel(GridDims g, int64_t c0, int64_t count, const void* buf, const uint32_t* links,
                              int mode, double* rho, double* u, int64_t out_stride)
{
   const int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
   if (k >= count) return;
   const int64_t c = c0 + k;
   int x, y, z;
   if (!cell_xyz(g, c, x, y, z)) return;
   const uint32_t lk = links ? links[c] : 0u;
   if (lk & kSolidBit) {
      const double nan = __longlong_as_double(0x7FF8000000000000LL);
      rho[k] = nan;
      u[k] = u[out_stride + k] = u[2 * out_stride + k] = nan;
      return;
   }
   double r = 0.0, m[3] = {0.0, 0.0, 0.0};
#pragma unroll
   for (int s = 0; s < Q; s++) {
      const double f = logical_pop<Q, ST>(g, buf, lk, x, y, z, c, s, mode);
      r += f;
#pragma unroll
      for (int d = 0; d < 3; d++) {
         const int cd = lat_c(Q, s, d);
         if (cd > 0) m[d] += f;
         else if (cd < 0) m[d] -= f;
      }
   }
   const double ir = 1.0 / r;
   rho[k] = r;
   u[k] = m[0] * ir;
   u[out_stride + k] = m[1] * ir;
   u[2 * out_stride + k] = m[2] * ir;
}

// FP64 mass / momentum sums over fluid cells, exact for physical states.
//
// A population f in [2^-32, 1) -- every population of a physical state -- is
// an integer multiple of 2^-84 below 1: its fixed-point image f * 2^84, the
// 53-bit significand shifted left by E - 991 (E the biased exponent, 991 for
// 2^-32), is exact.  The mass and momenta of such cells are therefore summed
// exactly, in 128-bit integers (below 2^84 * 27 * 2^31 < 2^120 in magnitude),
// so the totals do not depend on the order of the additions (block or grid
// shape) and are rounded only when converted to double at the end.  A cell
// with any population outside that range (zero, negative, 1 or more, NaN,
// Inf) is summed in FP64 instead, into separate accumulators whose per-block
// partials are added in a fixed order.  Zero stencil terms are left out and
// +-1 terms become adds or subtracts.
constexpr int kReduceThreads = 256;
constexpr uint32_t kFix84HiMin = (uint32_t)(1023 - 32) << 20;   // high word of 2^-32
constexpr uint32_t kFix84HiMax = (uint32_t)1023 << 20;          // high word of 1.0 (excluded)

// Fixed-point image f * 2^84 of a population in [2^-32, 1), at most 84 bits,
// as three 32-bit limbs: the 53-bit significand (21 bits in the high word)
// shifted left by E - 991, in [0, 31].
struct Fix84 {
   uint32_t w0, w1, w2;
};

__device__ __forceinline__ Fix84 fix84(double f)
{
   const uint32_t lo = (uint32_t)__double2loint(f), hi = (uint32_t)__double2hiint(f);
   const uint32_t mh = (hi & 0x000FFFFFu) | 0x00100000u;
   const uint32_t sh = (hi >> 20) - 991u;
   return {lo << sh, __funnelshift_l(lo, mh, sh), __funnelshift_l(mh, 0u, sh)};
}

// 128-bit two's-complement accumulator in four 32-bit limbs, added to with
// one carry chain per image.
struct Acc128 {
   uint32_t w[4];
};

__device__ __forceinline__ void acc_zero(Acc128& a) { a.w[0] = a.w[1] = a.w[2] = a.w[3] = 0u; }

__device__ __forceinline__ void acc_add(Acc128& a, const Fix84& x)
{
   asm("add.cc.u32 %0, %0, %4;\n\t"
       "addc.cc.u32 %1, %1, %5;\n\t"
       "addc.cc.u32 %2, %2, %6;\n\t"
       "addc.u32 %3, %3, 0;"
       : "+r"(a.w[0]), "+r"(a.w[1]), "+r"(a.w[2]), "+r"(a.w[3])
       : "r"(x.w0), "r"(x.w1), "r"(x.w2));
}

__device__ __forceinline__ void acc_sub(Acc128& a, const Fix84& x)
{
   asm("sub.cc.u32 %0, %0, %4;\n\t"
       "subc.cc.u32 %1, %1, %5;\n\t"
       "subc.cc.u32 %2, %2, %6;\n\t"
       "subc.u32 %3, %3, 0;"
       : "+r"(a.w[0]), "+r"(a.w[1]), "+r"(a.w[2]), "+r"(a.w[3])
       : "r"(x.w0), "r"(x.w1), "r"(x.w2));
}

__device__ __forceinline__ __int128 acc_value(const Acc128& a)
{
   const unsigned __int128 v = ((unsigned __int128)(((uint64_t)a.w[3] << 32) | a.w[2]) << 64) |
                               (((uint64_t)a.w[1] << 32) | a.w[0]);
   return (__int128)v;
}

struct ConservedAcc {
   Acc128 x[4];     // exact sums of the fixed-point cells, units of 2^-84
   double d[4];     // FP64 sums of the other cells
};

// One block's partial sums; the reduction scratch holds one per block.
struct ConservedPartial {
   __int128 x[4];
   double d[4];
};

__device__ __forceinline__ void conserved_zero(ConservedAcc& a)
{
#pragma unroll
   for (int k = 0; k < 4; k++) {
      acc_zero(a.x[k]);
      a.d[k] = 0.0;
   }
}

template <int Q>
__device__ __forceinline__ void conserved_add_cell(const double (&f)[Q], ConservedAcc& a)
{
   bool fixed = true;
#pragma unroll
   for (int s = 0; s < Q; s++) {
      const uint32_t hi = (uint32_t)__double2hiint(f[s]);
      fixed = fixed && (hi - kFix84HiMin) < (kFix84HiMax - kFix84HiMin);
   }
   if (fixed) {
#pragma unroll
      for (int s = 0; s < Q; s++) {
         const Fix84 X = fix84(f[s]);
         acc_add(a.x[0], X);
#pragma unroll
         for (int d = 0; d < 3; d++) {
            const int cd = lat_c(Q, s, d);
            if (cd > 0) acc_add(a.x[1 + d], X);
            else if (cd < 0) acc_sub(a.x[1 + d], X);
         }
      }
   } else {
      double r = 0.0, j[3] = {0.0, 0.0, 0.0};
#pragma unroll
      for (int s = 0; s < Q; s++) {
         r += f[s];
#pragma unroll
         for (int d = 0; d < 3; d++) {
            const int cd = lat_c(Q, s, d);
            if (cd > 0) j[d] += f[s];
            else if (cd < 0) j[d] -= f[s];
         }
      }
      a.d[0] += r;
#pragma unroll
      for (int d = 0; d < 3; d++) a.d[1 + d] += j[d];
   }
}

__device__ __forceinline__ __int128 shfl_down_i128(__int128 v, int off)
{
   const unsigned long long lo = __shfl_down_sync(0xFFFFFFFFu, (unsigned long long)v, off);
   const unsigned long long hi = __shfl_down_sync(0xFFFFFFFFu, (unsigned long long)((unsigned __int128)v >> 64), off);
   return (__int128)(((unsigned __int128)hi << 64) | lo);
}

// Reduce the block's accumulators (warp shuffles, then shared memory) into
// *out.  Every thread of the block must call it.
template <int NT>
__device__ __forceinline__ void conserved_block_store(const ConservedAcc& a, ConservedPartial* out)
{
   __shared__ __int128 shx[4][NT / 32];
   __shared__ double shd[4][NT / 32];
   const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
   for (int k = 0; k < 4; k++) {
      __int128 x = acc_value(a.x[k]);
      double d = a.d[k];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
         x += shfl_down_i128(x, off);
         d += __shfl_down_sync(0xFFFFFFFFu, d, off);
      }
      if (lane == 0) {
         shx[k][warp] = x;
         shd[k][warp] = d;
      }
   }
   __syncthreads();
   if (threadIdx.x < 4) {
      __int128 x = 0;
      double d = 0.0;
      for (int w = 0; w < NT / 32; w++) {
         x += shx[threadIdx.x][w];
         d += shd[threadIdx.x][w];
      }
      out->x[threadIdx.x] = x;
      out->d[threadIdx.x] = d;
   }
}

// The handle's reduction works plane by plane and needs no neighbour index.
// With M_r the sum of raw slot r over fluid cells and S_r the same with
// sign -1 where the cell's link bit r is set, the logical populations give
//   mass = sum_r M_r,
//   momentum_d = sum_r c_rd M_r (mode 0: slot s holds f_s),
//              = -sum_r c_rd M_r (mode 1: slot r holds f_opp(r) of its cell),
//              = sum_r c_rd S_r (mode 2, pull gather: slot r of cell n is
//                f_r of n + c_r when that neighbour is open, else bounced
//                back as f_opp(r) of n itself).
// Block b sums plane b mod Q over the cell range b / Q; consecutive blocks
// share a range, so its link words come from L2 after the first plane.
struct PlanePartial {
   __int128 m, s;   // exact sums, units of 2^-84
   double md, sd;   // FP64 sums of the elements outside [2^-32, 1)
};
constexpr int kPlaneRanges = 96;
constexpr int kPlaneUnroll = 4;

template <int Q, int ST>
__global__ void __launch_bounds__(kReduceThreads) conserved_plane_kernel(GridDims g, const void* buf,
                                                                        const uint32_t* links, int mode,
                                                                        int64_t per_range, PlanePartial* partials)
{
   const int r = (int)(blockIdx.x % Q);
   const int64_t c0 = (int64_t)(blockIdx.x / Q) * per_range;
   const int64_t c1 = c0 + per_range < g.ncell ? c0 + per_range : g.ncell;
   const double w = weight_at<Q>(r);
   const bool signed_links = mode == 2 && links != nullptr;
   Acc128 am, an;   // all elements; those with link bit r set (mode 2 only)
   acc_zero(am);
   acc_zero(an);
   double md = 0.0, nd = 0.0;
   for (int64_t cb = c0 + threadIdx.x; cb < c1; cb += (int64_t)kPlaneUnroll * blockDim.x) {
      uint32_t lk[kPlaneUnroll];
#pragma unroll
      for (int u = 0; u < kPlaneUnroll; u++) {
         const int64_t c = cb + (int64_t)u * blockDim.x;
         lk[u] = c < c1 ? (links ? links[c] : 0u) : kSolidBit;
      }
      double f[kPlaneUnroll];
#pragma unroll
      for (int u = 0; u < kPlaneUnroll; u++)
         f[u] = (lk[u] & kSolidBit) ? 0.0 : load_pop<ST>(buf, (int64_t)r * g.plane + cb + (int64_t)u * blockDim.x, w);
      bool rare = false;   // an element outside the fixed-point range
#pragma unroll
      for (int u = 0; u < kPlaneUnroll; u++) {
         if (lk[u] & kSolidBit) continue;
         const bool neg = signed_links && ((lk[u] >> r) & 1u);
         const uint32_t hi = (uint32_t)__double2hiint(f[u]);
         if ((hi - kFix84HiMin) < (kFix84HiMax - kFix84HiMin)) {
            const Fix84 X = fix84(f[u]);
            acc_add(am, X);
            if (neg) acc_add(an, X);
         } else {
            rare = true;
         }
      }
      // The FP64 adds sit behind a warp-uniform branch: predicated off, they
      // would still occupy the (slow) FP64 pipe on every element.
      if (__any_sync(__activemask(), rare)) {
#pragma unroll
         for (int u = 0; u < kPlaneUnroll; u++) {
            if (lk[u] & kSolidBit) continue;
            const uint32_t hi = (uint32_t)__double2hiint(f[u]);
            if ((hi - kFix84HiMin) < (kFix84HiMax - kFix84HiMin)) continue;
            md += f[u];
            if (signed_links && ((lk[u] >> r) & 1u)) nd += f[u];
         }
      }
   }
   __shared__ __int128 shx[2][kReduceThreads / 32];
   __shared__ double shd[2][kReduceThreads / 32];
   const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   // signed sums: all minus twice the flipped ones
   __int128 m = acc_value(am), sg = m - 2 * acc_value(an);
   double sd = md - 2.0 * nd;
#pragma unroll
   for (int off = 16; off > 0; off >>= 1) {
      m += shfl_down_i128(m, off);
      sg += shfl_down_i128(sg, off);
      md += __shfl_down_sync(0xFFFFFFFFu, md, off);
      sd += __shfl_down_sync(0xFFFFFFFFu, sd, off);
   }
   if (lane == 0) {
      shx[0][warp] = m;
      shx[1][warp] = sg;
      shd[0][warp] = md;
      shd[1][warp] = sd;
   }
   __syncthreads();
   if (threadIdx.x == 0) {
      PlanePartial pp{0, 0, 0.0, 0.0};
      for (int k = 0; k < kReduceThreads / 32; k++) {
         pp.m += shx[0][k];
         pp.s += shx[1][k];
         pp.md += shd[0][k];
         pp.sd += shd[1][k];
      }
      partials[blockIdx.x] = pp;
   }
}

// Cells per range of conserved_plane_kernel (a multiple of the unrolled
// block stride) and the number of blocks it launches.
inline int64_t plane_per_range(int64_t ncell)
{
   const int64_t step = (int64_t)kPlaneUnroll * kReduceThreads;
   int64_t per = (ncell + kPlaneRanges - 1) / kPlaneRanges;
   return (per + step - 1) / step * step;
}
inline int plane_blocks(int Q, int64_t ncell)
{
   return Q * (int)((ncell + plane_per_range(ncell) - 1) / plane_per_range(ncell));
}

// Nearest double to v (to within one rounding of the low word).
__device__ __forceinline__ double i128_to_double(__int128 v)
{
   const bool neg = v < 0;
   const unsigned __int128 m = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
   const double d = __ull2double_rn((unsigned long long)(m >> 64)) * 0x1p64 + __ull2double_rn((unsigned long long)m);
   return neg ? -d : d;
}

// static: every translation unit that includes this header gets its own copy.
static __global__ void conserved_final_kernel(const ConservedPartial* partials, int nblocks, double* out)
{
   __shared__ __int128 shx[4][kReduceThreads];
   __shared__ double shd[4][kReduceThreads];
   for (int k = 0; k < 4; k++) {
      __int128 x = 0;
      double d = 0.0;
      for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
         x += partials[b].x[k];
         d += partials[b].d[k];
      }
      shx[k][threadIdx.x] = x;
      shd[k][threadIdx.x] = d;
   }
   __syncthreads();
   for (int stride = blockDim.x / 2; stride > 0; stride >>= 1) {
      if ((int)threadIdx.x < stride)
         for (int k = 0; k < 4; k++) {
            shx[k][threadIdx.x] += shx[k][threadIdx.x + stride];
            shd[k][threadIdx.x] += shd[k][threadIdx.x + stride];
         }
      __syncthreads();
   }
   if (threadIdx.x < 4) out[threadIdx.x] = i128_to_double(shx[threadIdx.x][0]) * 0x1p-84 + shd[threadIdx.x][0];
}

// Totals from the plane partials of conserved_plane_kernel (nblocks of
// them, plane b mod Q): out = {mass, momentum x, y, z}.
template <int Q>
__global__ void conserved_plane_final_kernel(const PlanePartial* partials, int nblocks, int mode, double* out)
{
   __shared__ __int128 shx[4][kReduceThreads];
   __shared__ double shd[4][kReduceThreads];
   __int128 x[4] = {0, 0, 0, 0};
   double d[4] = {0.0, 0.0, 0.0, 0.0};
   for (int b = threadIdx.x; b < nblocks; b += blockDim.x) {
      const int r = b % Q;
      const PlanePartial pp = partials[b];
      x[0] += pp.m;
      d[0] += pp.md;
      // mode 2 uses the signed sums; mode 1 flips every direction
      const __int128 xm = mode == 2 ? pp.s : pp.m;
      const double dm = mode == 2 ? pp.sd : pp.md;
#pragma unroll
      for (int e = 0; e < 3; e++) {
         const int cr = (mode == 1 ? -1 : 1) * velocity_at<Q>(r, e);
         if (cr > 0) {
            x[1 + e] += xm;
            d[1 + e] += dm;
         } else if (cr < 0) {
            x[1 + e] -= xm;
            d[1 + e] -= dm;
         }
      }
   }
#pragma unroll
   for (int k = 0; k < 4; k++) {
      shx[k][threadIdx.x] = x[k];
      shd[k][threadIdx.x] = d[k];
   }
   __syncthreads();
   for (int stride = blockDim.x / 2; stride > 0; stride >>= 1) {
      if ((int)threadIdx.x < stride)
         for (int k = 0; k < 4; k++) {
            shx[k][threadIdx.x] += shx[k][threadIdx.x + stride];
            shd[k][threadIdx.x] += shd[k][threadIdx.x + stride];
         }
      __syncthreads();
   }
   if (threadIdx.x < 4) out[threadIdx.x] = i128_to_double(shx[threadIdx.x][0]) * 0x1p-84 + shd[threadIdx.x][0];
}

}  // namespace lbm
