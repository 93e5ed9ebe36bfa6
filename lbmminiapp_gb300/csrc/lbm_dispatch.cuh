// Launch dispatch for the step kernels: one translation unit per lattice and
// storage group instantiates its kernels (lbm_step_q*.cu), so the library
// builds in parallel.
#pragma once

#include <cuda_runtime.h>

#include "lbm_step.cuh"
#include "lbm_step_async.cuh"
#include "lbm_step_async_low.cuh"

namespace lbm {

struct Launch {
   dim3 grid, block;
   cudaStream_t stream;
   bool idx32;   // plane stride below 2^32 bytes: 32-bit stride arithmetic
   bool pair;    // two cells per thread (shifted storage, periodic box, even nx, full grid)
   dim3 pair_grid, pair_block;
   bool async;   // pipelined persistent kernel (FP64 storage, F64X, full grid, 32-bit plane stride)
   bool async_low;   // pipelined persistent kernel for shifted storage (full grid, 32-bit plane stride)
   AsyncGeom ag;
};

template <int Q, int ST, int AR, int KIND>
cudaError_t launch_kind(const Launch& L, const KParams& p, const void* src, void* dst, bool links,
                        bool fields)
{
   using T = typename Store<ST>::T;
   const T* s = static_cast<const T*>(src);
   T* d = static_cast<T*>(dst);
   if constexpr (ST != ST_F64) {
      if (L.pair && !links && !fields) {
         if (L.idx32)
            return launch_overlapped(step_pair_kernel<Q, ST, KIND, uint32_t>, L.pair_grid, L.pair_block, 0, L.stream,
                                     p, s, d);
         return launch_overlapped(step_pair_kernel<Q, ST, KIND, int64_t>, L.pair_grid, L.pair_block, 0, L.stream, p,
                                  s, d);
      }
      if (L.async_low && links && !fields) {
         const bool ragged = p.nx % 32 != 0;
         return ragged ? launch_async_low<Q, ST, KIND, true, true>(p, L.ag, src, dst, L.stream)
                       : launch_async_low<Q, ST, KIND, true, false>(p, L.ag, src, dst, L.stream);
      }
   }
   if constexpr (ST == ST_F64 && AR == AR_F64X) {
      if (L.async && !fields) {
         const bool ragged = p.nx % 32 != 0;
         if (links) return ragged ? launch_async<Q, KIND, true, true>(p, L.ag, src, dst, L.stream)
                                  : launch_async<Q, KIND, true, false>(p, L.ag, src, dst, L.stream);
         return ragged ? launch_async<Q, KIND, false, true>(p, L.ag, src, dst, L.stream)
                       : launch_async<Q, KIND, false, false>(p, L.ag, src, dst, L.stream);
      }
   }
   // Per-cell fields always use the exact FP64 arithmetic when FP64 is stored.
   constexpr int ARF = (AR == AR_F64X) ? AR_F64 : AR;
   // Per-cell fields (porosity, force field): 64-bit stride arithmetic only.
   // The plain step kernels get a 32-bit stride variant for planes below 4 GiB.
   if (fields) {
      if (links)
         return launch_overlapped(step_kernel<Q, ST, ARF, KIND, true, true, int64_t>, L.grid, L.block, 0, L.stream, p,
                                  s, d);
      return launch_overlapped(step_kernel<Q, ST, ARF, KIND, false, true, int64_t>, L.grid, L.block, 0, L.stream, p, s,
                               d);
   }
   if (L.idx32) {
      if (links)
         return launch_overlapped(step_kernel<Q, ST, AR, KIND, true, false, uint32_t>, L.grid, L.block, 0, L.stream, p,
                                  s, d);
      return launch_overlapped(step_kernel<Q, ST, AR, KIND, false, false, uint32_t>, L.grid, L.block, 0, L.stream, p,
                               s, d);
   }
   if (links)
      return launch_overlapped(step_kernel<Q, ST, AR, KIND, true, false, int64_t>, L.grid, L.block, 0, L.stream, p, s,
                               d);
   return launch_overlapped(step_kernel<Q, ST, AR, KIND, false, false, int64_t>, L.grid, L.block, 0, L.stream, p, s,
                            d);
}

template <int Q, int ST, int AR>
cudaError_t launch_step_t(int kind, const Launch& L, const KParams& p, const void* src, void* dst,
                          bool links, bool fields)
{
   switch (kind) {
      case K_AA_EVEN: return launch_kind<Q, ST, AR, K_AA_EVEN>(L, p, src, dst, links, fields);
      case K_AA_ODD: return launch_kind<Q, ST, AR, K_AA_ODD>(L, p, src, dst, links, fields);
      case K_AB_PUSH: return launch_kind<Q, ST, AR, K_AB_PUSH>(L, p, src, dst, links, fields);
      default: return launch_kind<Q, ST, AR, K_AB_PULL>(L, p, src, dst, links, fields);
   }
}

// Defined in lbm_step_q19_f64.cu, lbm_step_q19_low.cu, lbm_step_q27_f64.cu,
// lbm_step_q27_low.cu.
cudaError_t launch_step_q19_f64(int arith, int kind, const Launch& L, const KParams& p,
                                const void* src, void* dst, bool links, bool fields);
cudaError_t launch_step_q19_low(int storage, int kind, const Launch& L, const KParams& p,
                                const void* src, void* dst, bool links, bool fields);
cudaError_t launch_step_q27_f64(int arith, int kind, const Launch& L, const KParams& p,
                                const void* src, void* dst, bool links, bool fields);
cudaError_t launch_step_q27_low(int storage, int kind, const Launch& L, const KParams& p,
                                const void* src, void* dst, bool links, bool fields);

}  // namespace lbm
