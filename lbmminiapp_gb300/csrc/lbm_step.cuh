// Fused collide-stream step kernels.
//
// One thread per cell along the contiguous x axis; a 3-D grid
// (x blocks, y, z) so no per-thread division is needed.  Population buffers
// are planar: direction s of cell c lives at s*plane + c.
//
// Streaming replaces the reference's int32 adjacency list
// (src/geometries/GeometryAAAB.cpp:18-124) with index arithmetic: the
// neighbour x +- c_s wraps on periodic axes, and a per-cell 32-bit link word
// (present only when the geometry has solids or non-periodic faces) says
// which neighbours bounce back to the own cell's opposite slot.
//
//   AA even  (KernelAA_SOA_Base.cpp:173-254): read own slot opp(s), write own slot s
//   AA odd   (KernelAA_SOA_Base.cpp:257-342): read slot s at x - c_s (or own slot opp(s)),
//            write slot opp(s) at x + c_s (or own slot s)
//   AB push  (KernelAB_SOA_Base.cpp:111-186): read own slot s from src, write slot s at
//            x + c_s (or own slot opp(s)) in tgt
//   AB pull  (KernelAB_SOA_Pull.cpp:113-194): read slot s at x - c_s (or own slot opp(s))
//            from src, write own slot s in tgt
#pragma once

#include "lbm_f64x.cuh"
#include "lbm_launch.cuh"
#include "lbm_physics.cuh"

namespace lbm {

// IT is uint32_t when a plane is below 4 GiB (32-bit stride arithmetic),
// int64_t otherwise.  Cell indices and neighbour offsets always fit 32 bits
// (fewer than 2^31 cells per handle).
struct CellIndex {
   int64_t c;
   int dxm, dxp, dym, dyp, dzm, dzp;   // neighbour offsets in cells
};

__device__ __forceinline__ bool cell_of_thread(const KParams& p, CellIndex& ci)
{
   const int x = blockIdx.x * blockDim.x + threadIdx.x;
   const int y = blockIdx.y;
   const int z = p.z0 + blockIdx.z;
   if (x >= p.nx) return false;
   const int64_t row = (int64_t)z * p.ny + y;
   ci.c = row * p.nx + x;
   if (ci.c < p.cstart || ci.c >= p.cend) return false;
   ci.dxm = (x == 0) ? p.nx - 1 : -1;
   ci.dxp = (x == p.nx - 1) ? -(p.nx - 1) : 1;
   ci.dym = (y == 0) ? (p.ny - 1) * p.nx : -p.nx;
   ci.dyp = (y == p.ny - 1) ? -(p.ny - 1) * p.nx : p.nx;
   const int nxy = p.nx * p.ny;
   ci.dzm = (z == 0) ? (p.nz - 1) * nxy : -nxy;
   ci.dzp = (z == p.nz - 1) ? -(p.nz - 1) * nxy : nxy;
   return true;
}

// Cell index of x + (sx, sy, sz) with periodic wrap on every axis (a wrapped
// neighbour across a non-periodic face is always flagged in the link word and
// never dereferenced).
__device__ __forceinline__ int nbr_off(const CellIndex& ci, int sx, int sy, int sz)
{
   int off = 0;
   if (sx > 0) off += ci.dxp; else if (sx < 0) off += ci.dxm;
   if (sy > 0) off += ci.dyp; else if (sy < 0) off += ci.dym;
   if (sz > 0) off += ci.dzp; else if (sz < 0) off += ci.dzm;
   return off;
}

// Access to slot `slot` of the cell at offset `off` (in cells, small and
// signed) from this thread's cell: byte address = cell base + slot * plane
// bytes + off * element bytes.  With IT = uint32_t the plane stride in bytes
// fits 32 bits and slot * stride is one 32x32->64 multiply-add.
struct Access {
   int slot;
   int off;
};

template <int Q, int KIND, bool LINKS>
__device__ __forceinline__ Access read_access(const CellIndex& ci, uint32_t lk, int s)
{
   const int o = lat_opp(Q, s);
   if (KIND == K_AA_EVEN) return {o, 0};
   if (KIND == K_AB_PUSH || s == lat_rest(Q)) return {s, 0};
   // AA odd, AB pull: slot s at x - c_s unless that neighbour is blocked.
   if (LINKS && ((lk >> o) & 1u)) return {o, 0};
   return {s, nbr_off(ci, -lat_c(Q, s, 0), -lat_c(Q, s, 1), -lat_c(Q, s, 2))};
}

template <int Q, int KIND, bool LINKS>
__device__ __forceinline__ Access write_access(const CellIndex& ci, uint32_t lk, int s)
{
   const int o = lat_opp(Q, s);
   if (KIND == K_AA_EVEN || KIND == K_AB_PULL || s == lat_rest(Q)) return {s, 0};
   const bool blocked = LINKS && ((lk >> s) & 1u);
   if (KIND == K_AA_ODD) {
      if (blocked) return {s, 0};
      return {o, nbr_off(ci, lat_c(Q, s, 0), lat_c(Q, s, 1), lat_c(Q, s, 2))};
   }
   // AB push
   if (blocked) return {o, 0};
   return {s, nbr_off(ci, lat_c(Q, s, 0), lat_c(Q, s, 1), lat_c(Q, s, 2))};
}

// write_access for a non-rest direction s known at run time (o = opp(s),
// velocity (cx, cy, cz)).
template <int KIND, bool LINKS>
__device__ __forceinline__ Access write_access_rt(const CellIndex& ci, uint32_t lk, int s, int o, int cx, int cy, int cz)
{
   if (KIND == K_AA_EVEN || KIND == K_AB_PULL) return {s, 0};
   const bool blocked = LINKS && ((lk >> s) & 1u);
   if (KIND == K_AA_ODD) return blocked ? Access{s, 0} : Access{o, nbr_off(ci, cx, cy, cz)};
   return blocked ? Access{o, 0} : Access{s, nbr_off(ci, cx, cy, cz)};
}

template <typename T, typename IT>
__device__ __forceinline__ T* slot_ptr(T* cell_base, IT plane_bytes, Access a)
{
   const uintptr_t p = reinterpret_cast<uintptr_t>(cell_base) + (uint64_t)(uint32_t)a.slot * (uint64_t)plane_bytes;
   return reinterpret_cast<T*>(p) + a.off;
}

template <bool FIELDS>
__device__ __forceinline__ void cell_force_f64(const KParams& p, int64_t c, double& F0, double& F1,
                                               double& F2, double& sp)
{
   F0 = p.F[0]; F1 = p.F[1]; F2 = p.F[2]; sp = 0.0;
   if (FIELDS) {
      if (p.force_field) {
         F0 = __dadd_rn(F0, p.force_field[c]);
         F1 = __dadd_rn(F1, p.force_field[p.plane + c]);
         F2 = __dadd_rn(F2, p.force_field[2 * p.plane + c]);
      }
      if (p.porosity) sp = p.porosity[c];
   }
}

template <bool FIELDS>
__device__ __forceinline__ void cell_force_f32(const KParams& p, int64_t c, float& F0, float& F1,
                                               float& F2, float& sp)
{
   F0 = p.Ff[0]; F1 = p.Ff[1]; F2 = p.Ff[2]; sp = 0.0f;
   if (FIELDS) {
      if (p.force_field_f) {
         F0 += p.force_field_f[c];
         F1 += p.force_field_f[p.plane + c];
         F2 += p.force_field_f[2 * p.plane + c];
      }
      if (p.porosity_f) sp = p.porosity_f[c];
   }
}

// One launch = one time step (or one range of it) of one propagation kind.
template <int Q, int ST, int AR, int KIND, bool LINKS, bool FIELDS, typename IT>
__global__ void __launch_bounds__(256) step_kernel(const KParams p, const typename Store<ST>::T* src,
                                                   typename Store<ST>::T* dst)
{
   wait_prior_grid();
   CellIndex ci;
   if (!cell_of_thread(p, ci)) return;
   uint32_t lk = 0;
   if (LINKS) {
      lk = p.links[ci.c];
      if (lk & kSolidBit) return;
   }
   using T = typename Store<ST>::T;
   const IT pb = (IT)p.plane * (IT)sizeof(T);
   const T* sbase = src + ci.c;
   T* dbase = dst + ci.c;
   if constexpr (AR == AR_F64) {
      double d[Q], o[Q];
#pragma unroll
      for (int s = 0; s < Q; s++) d[s] = *slot_ptr(sbase, pb, read_access<Q, KIND, LINKS>(ci, lk, s));
      double F0, F1, F2, sp;
      cell_force_f64<FIELDS>(p, ci.c, F0, F1, F2, sp);
      collide_f64<Q>(d, o, F0, F1, F2, sp, p);
#pragma unroll
      for (int s = 0; s < Q; s++) *slot_ptr(dbase, pb, write_access<Q, KIND, LINKS>(ci, lk, s)) = o[s];
   } else if constexpr (AR == AR_F64X) {
      uint64_t bits[Q];
      const unsigned long long* s64 = reinterpret_cast<const unsigned long long*>(sbase);
#pragma unroll
      for (int s = 0; s < Q; s++) bits[s] = *slot_ptr(s64, pb, read_access<Q, KIND, LINKS>(ci, lk, s));
      static_assert(!FIELDS, "per-cell fields use the exact FP64 arithmetic");
      collide_f64x<Q>(bits, p);
      unsigned long long* d64 = reinterpret_cast<unsigned long long*>(dbase);
#pragma unroll
      for (int s = 0; s < Q; s++) *slot_ptr(d64, pb, write_access<Q, KIND, LINKS>(ci, lk, s)) = bits[s];
   } else {
      float g[Q], o[Q];
#pragma unroll
      for (int s = 0; s < Q; s++) g[s] = load_raw(slot_ptr(sbase, pb, read_access<Q, KIND, LINKS>(ci, lk, s)));
      float F0, F1, F2, sp;
      cell_force_f32<FIELDS>(p, ci.c, F0, F1, F2, sp);
      if (FIELDS || p.forced) collide_f32<Q, ST, true>(g, o, F0, F1, F2, sp, p);
      else collide_f32<Q, ST, false>(g, o, F0, F1, F2, sp, p);
#pragma unroll
      for (int s = 0; s < Q; s++) store_raw(slot_ptr(dbase, pb, write_access<Q, KIND, LINKS>(ci, lk, s)), o[s]);
   }
}

// ------------------------------------------------------------------------
// Two cells per thread (x0, x0+1) for shifted FP32/BF16/FP16 storage in a
// fully periodic box: planes not shifted along x are read and written as one
// aligned 2-element vector (half2 / bfloat162 / float2); x-shifted planes use
// two scalar accesses.  Requires an even nx and a full-grid launch.
template <typename T> struct PairVec;
template <> struct PairVec<float> {
   using V = float2;
   __device__ static float2 get(V v) { return v; }
   __device__ static V put(float a, float b) { return make_float2(a, b); }
};
template <> struct PairVec<__half> {
   using V = __half2;
   __device__ static float2 get(V v) { return __half22float2(v); }
   __device__ static V put(float a, float b) { return __floats2half2_rn(a, b); }
};
template <> struct PairVec<__nv_bfloat16> {
   using V = __nv_bfloat162;
   __device__ static float2 get(V v) { return __bfloat1622float2(v); }
   __device__ static V put(float a, float b) { return __floats2bfloat162_rn(a, b); }
};

__device__ __forceinline__ void cell_offsets(const KParams& p, int x, int y, int z, CellIndex& ci)
{
   ci.c = ((int64_t)z * p.ny + y) * p.nx + x;
   ci.dxm = (x == 0) ? p.nx - 1 : -1;
   ci.dxp = (x == p.nx - 1) ? -(p.nx - 1) : 1;
   ci.dym = (y == 0) ? (p.ny - 1) * p.nx : -p.nx;
   ci.dyp = (y == p.ny - 1) ? -(p.ny - 1) * p.nx : p.nx;
   const int nxy = p.nx * p.ny;
   ci.dzm = (z == 0) ? (p.nz - 1) * nxy : -nxy;
   ci.dzp = (z == p.nz - 1) ? -(p.nz - 1) * nxy : nxy;
}

template <int Q, int KIND>
__device__ constexpr bool read_shifted_x(int s)
{
   return (KIND == K_AA_ODD || KIND == K_AB_PULL) && s != lat_rest(Q) && lat_c(Q, s, 0) != 0;
}

template <int Q, int KIND>
__device__ constexpr bool write_shifted_x(int s)
{
   return (KIND == K_AA_ODD || KIND == K_AB_PUSH) && s != lat_rest(Q) && lat_c(Q, s, 0) != 0;
}

// Resident blocks per SM: the kernel waits on its loads, and more resident
// warps keep more of them in flight.  D3Q19 16-bit storage: four blocks (at
// most 64 registers; measured on GB300, FP16 71 -> 76 GLUPS at 512^3); D3Q19
// FP32: three; D3Q27: two (fewer registers would spill).
template <int Q, int ST>
constexpr int pair_min_blocks() { return Q == 27 ? 2 : (Store<ST>::bytes == 2 ? 4 : 3); }

template <int Q, int ST, int KIND, typename IT>
__global__ void __launch_bounds__(256, pair_min_blocks<Q, ST>()) step_pair_kernel(const KParams p, const typename Store<ST>::T* src,
                                                        typename Store<ST>::T* dst)
{
   using T = typename Store<ST>::T;
   using PV = PairVec<T>;
   wait_prior_grid();
   const int x0 = 2 * (blockIdx.x * blockDim.x + threadIdx.x);
   if (x0 >= p.nx) return;
   const int y = blockIdx.y, z = p.z0 + blockIdx.z;
   CellIndex c0, c1;
   cell_offsets(p, x0, y, z, c0);
   cell_offsets(p, x0 + 1, y, z, c1);
   const IT pb = (IT)p.plane * (IT)sizeof(T);
   const T* s0 = src + c0.c;
   const T* s1 = src + c1.c;
   T* d0 = dst + c0.c;
   T* d1 = dst + c1.c;
   float g0[Q], g1[Q], o0[Q], o1[Q];
#pragma unroll
   for (int s = 0; s < Q; s++) {
      const Access a0 = read_access<Q, KIND, false>(c0, 0u, s);
      if (read_shifted_x<Q, KIND>(s)) {
         const Access a1 = read_access<Q, KIND, false>(c1, 0u, s);
         g0[s] = load_raw(slot_ptr(s0, pb, a0));
         g1[s] = load_raw(slot_ptr(s1, pb, a1));
      } else {
         const float2 v = PV::get(*reinterpret_cast<const typename PV::V*>(slot_ptr(s0, pb, a0)));
         g0[s] = v.x;
         g1[s] = v.y;
      }
   }
   if (p.forced) {
      collide_f32<Q, ST, true>(g0, o0, p.Ff[0], p.Ff[1], p.Ff[2], 0.0f, p);
      collide_f32<Q, ST, true>(g1, o1, p.Ff[0], p.Ff[1], p.Ff[2], 0.0f, p);
   } else {
      collide_f32<Q, ST, false>(g0, o0, 0.0f, 0.0f, 0.0f, 0.0f, p);
      collide_f32<Q, ST, false>(g1, o1, 0.0f, 0.0f, 0.0f, 0.0f, p);
   }
#pragma unroll
   for (int s = 0; s < Q; s++) {
      const Access a0 = write_access<Q, KIND, false>(c0, 0u, s);
      if (write_shifted_x<Q, KIND>(s)) {
         const Access a1 = write_access<Q, KIND, false>(c1, 0u, s);
         store_raw(slot_ptr(d0, pb, a0), o0[s]);
         store_raw(slot_ptr(d1, pb, a1), o1[s]);
      } else {
         *reinterpret_cast<typename PV::V*>(slot_ptr(d0, pb, a0)) = PV::put(o0[s], o1[s]);
      }
   }
}

}  // namespace lbm
