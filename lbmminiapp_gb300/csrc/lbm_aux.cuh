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
template <int Q, int ST>
__global__ void export_plane_kernel(GridDims g, const void* buf, const uint32_t* links, int s, int mode,
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
   const int o = lat_opp(Q, s);
   int64_t idx;
   int slot;
   if (mode == 0) {
      slot = s;
      idx = (int64_t)s * g.plane + c;
   } else if (mode == 1 || s == lat_rest(Q) || ((lk >> o) & 1u)) {
      slot = o;
      idx = (int64_t)o * g.plane + c;
   } else {
      slot = s;
      const int64_t n = nbr_cell(g, x, y, z, -lat_c(Q, s, 0), -lat_c(Q, s, 1), -lat_c(Q, s, 2));
      idx = (int64_t)s * g.plane + n;
   }
   dst[c] = load_pop<ST>(buf, idx, lat_w(Q, slot));
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

// FP64 mass / momentum sums over fluid cells.  Each block reduces its cells
// with warp shuffles and shared memory and writes one partial (4 doubles) to
// `partials`; conserved_final_kernel adds the partials in a fixed order, so the
// result does not depend on scheduling.
constexpr int kReduceThreads = 256;

template <int Q, int ST>
__global__ void __launch_bounds__(kReduceThreads) conserved_partial_kernel(GridDims g, const void* buf,
                                                                          const uint32_t* links, int mode,
                                                                          double* partials)
{
   double acc[4] = {0.0, 0.0, 0.0, 0.0};
   for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < g.ncell;
        c += (int64_t)gridDim.x * blockDim.x) {
      int x, y, z;
      cell_xyz(g, c, x, y, z);
      const uint32_t lk = links ? links[c] : 0u;
      if (lk & kSolidBit) continue;
#pragma unroll
      for (int s = 0; s < Q; s++) {
         const double f = logical_pop<Q, ST>(g, buf, lk, x, y, z, c, s, mode);
         acc[0] += f;
         acc[1] += f * lat_c(Q, s, 0);
         acc[2] += f * lat_c(Q, s, 1);
         acc[3] += f * lat_c(Q, s, 2);
      }
   }
   __shared__ double sh[4][kReduceThreads / 32];
   const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
   for (int k = 0; k < 4; k++) {
      double v = acc[k];
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, off);
      if (lane == 0) sh[k][warp] = v;
   }
   __syncthreads();
   if (threadIdx.x < 4) {
      double v = 0.0;
      for (int w = 0; w < kReduceThreads / 32; w++) v += sh[threadIdx.x][w];
      partials[(int64_t)blockIdx.x * 4 + threadIdx.x] = v;
   }
}

// static: every translation unit that includes this header gets its own copy.
static __global__ void conserved_final_kernel(const double* partials, int nblocks, double* out)
{
   __shared__ double sh[4][kReduceThreads];
   for (int k = 0; k < 4; k++) {
      double v = 0.0;
      for (int b = threadIdx.x; b < nblocks; b += blockDim.x) v += partials[(int64_t)b * 4 + k];
      sh[k][threadIdx.x] = v;
   }
   __syncthreads();
   for (int stride = blockDim.x / 2; stride > 0; stride >>= 1) {
      if ((int)threadIdx.x < stride)
         for (int k = 0; k < 4; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + stride];
      __syncthreads();
   }
   if (threadIdx.x < 4) out[threadIdx.x] = sh[threadIdx.x][0];
}

}  // namespace lbm
