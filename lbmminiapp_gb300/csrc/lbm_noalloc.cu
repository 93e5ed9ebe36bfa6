// lbm_reduce_conserved_noalloc: the FP64 mass / momentum reduction for callers
// that cannot allocate device memory.
//
// Some hosts of this library cannot call cudaMalloc once they are running:
// codes that hand every device byte to their own pool or arena at start-up,
// and drivers that must not allocate inside their time loop.  They already own
// the population buffer and the output, so this entry point takes everything
// as caller-owned device memory and keeps its only scratch -- one FP64 partial
// sum per block -- in a file-scope device array instead of an allocation.
//
// The sums are the handle reduction's (exact 128-bit fixed-point sums for
// cells whose populations lie in [2^-32, 1), FP64 for the others).  The
// scratch array holds kNoAllocMaxBlocks partials (96 bytes each, 384 KiB)
// and lives on every GPU that loads the library until the process exits.
// One block reduces a run of consecutive cells, at least kNoAllocMinCells
// and as many as keep the block count within kNoAllocMaxBlocks; the entry
// point accepts at most 2^28 cells and rejects larger grids.  Every call
// shares the array; each launch writes every partial its final pass reads, so
// nothing needs clearing, but two calls that overlap on the GPU (different
// streams, no ordering) race on it.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "../../include/lbm_gb300.h"
#include "lbm_aux.cuh"

using namespace lbm;

namespace {

constexpr int kNoAllocThreads = 256;
constexpr int kNoAllocMaxBlocks = 4096;
constexpr int64_t kNoAllocMinCells = 4096;
constexpr int64_t kNoAllocMaxCells = (int64_t)1 << 28;
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) ConservedPartial g_noalloc_partials[kNoAllocMaxBlocks];

// Device address of g_noalloc_partials per device ordinal, looked up once per
// device with that device current (host code must not use the symbol itself).
ConservedPartial* g_scratch_addr[kNoAllocMaxDevices] = {};
std::mutex g_scratch_mutex;

// Direction s of cell (x, y, z) with the slot convention `mode` (0: slot s,
// 1: own slot opp(s), 2: pull gather) and bounce-back taken from the solid
// mask and the non-periodic faces.
template <int Q, int ST>
__device__ __forceinline__ double logical_pop_mask(const GridDims& g, const void* buf, const uint8_t* solid,
                                                   int x, int y, int z, int64_t c, int s, int mode)
{
   const int o = lat_opp(Q, s);
   if (mode == 0) return load_pop<ST>(buf, (int64_t)s * g.plane + c, lat_w(Q, s));
   if (mode == 1 || s == lat_rest(Q)) return load_pop<ST>(buf, (int64_t)o * g.plane + c, lat_w(Q, o));
   const int64_t n = nbr_cell(g, x, y, z, -lat_c(Q, s, 0), -lat_c(Q, s, 1), -lat_c(Q, s, 2));
   if (n < 0 || (solid && solid[n])) return load_pop<ST>(buf, (int64_t)o * g.plane + c, lat_w(Q, o));
   return load_pop<ST>(buf, (int64_t)s * g.plane + n, lat_w(Q, s));
}

// Block b reduces the cells [b * per_block, (b + 1) * per_block).
template <int Q, int ST>
__global__ void __launch_bounds__(kNoAllocThreads) conserved_chunk_kernel(GridDims g, const void* buf,
                                                                          const uint8_t* solid, int mode,
                                                                          int64_t per_block,
                                                                          ConservedPartial* partials)
{
   ConservedAcc acc;
   conserved_zero(acc);
   const int64_t begin = (int64_t)blockIdx.x * per_block;
   const int64_t end = begin + per_block < g.ncell ? begin + per_block : g.ncell;
   for (int64_t c = begin + threadIdx.x; c < end; c += blockDim.x) {
      if (solid && solid[c]) continue;
      int x, y, z;
      cell_xyz(g, c, x, y, z);
      double f[Q];
#pragma unroll
      for (int s = 0; s < Q; s++) f[s] = logical_pop_mask<Q, ST>(g, buf, solid, x, y, z, c, s, mode);
      conserved_add_cell<Q>(f, acc);
   }
   conserved_block_store<kNoAllocThreads>(acc, partials + blockIdx.x);
}

template <int Q, int ST>
cudaError_t launch_chunks(const GridDims& g, const void* buf, const uint8_t* solid, int mode,
                          ConservedPartial* scratch, int64_t per_block, int nblocks, cudaStream_t st)
{
   conserved_chunk_kernel<Q, ST><<<nblocks, kNoAllocThreads, 0, st>>>(g, buf, solid, mode, per_block, scratch);
   return cudaGetLastError();
}

lbm_status noalloc_fail(lbm_status s, const char* msg)
{
   fprintf(stderr, "lbm_reduce_conserved_noalloc: %s\n", msg);
   return s;
}

}  // namespace

extern "C" lbm_status lbm_reduce_conserved_noalloc(int lattice, int storage, int nx, int ny, int nz,
                                                   int64_t plane_stride, const void* dstrb,
                                                   const uint8_t* solid, const int periodic[3], int readout,
                                                   double* out, void* stream)
{
   if ((lattice != 19 && lattice != 27) || storage < LBM_STORE_F64 || storage > LBM_STORE_F16)
      return noalloc_fail(LBM_ERR_INVALID_ARGUMENT, "lattice must be 19 or 27 and storage an LBM_STORE_*");
   if (nx < 1 || ny < 1 || nz < 1 || !dstrb || !out || !periodic || readout < 0 || readout > 2)
      return noalloc_fail(LBM_ERR_INVALID_ARGUMENT, "bad grid, pointer or readout mode");
   const int64_t ncell = (int64_t)nx * ny * nz;
   if (ncell > kNoAllocMaxCells)
      return noalloc_fail(LBM_ERR_INVALID_ARGUMENT,
                          "grid exceeds the static scratch: at most 268435456 cells (2^28)");
   if (plane_stride < ncell) return noalloc_fail(LBM_ERR_INVALID_ARGUMENT, "plane_stride below nx*ny*nz");

   int dev = 0;
   cudaError_t e = cudaGetDevice(&dev);
   if (e != cudaSuccess) return noalloc_fail(LBM_ERR_CUDA, cudaGetErrorString(e));
   if (dev < 0 || dev >= kNoAllocMaxDevices) return noalloc_fail(LBM_ERR_UNSUPPORTED, "device ordinal above 63");
   ConservedPartial* scratch = nullptr;
   {
      std::lock_guard<std::mutex> lock(g_scratch_mutex);
      if (!g_scratch_addr[dev]) {
         // Set-up, once per device, with that device current.
         e = cudaGetSymbolAddress((void**)&g_scratch_addr[dev], g_noalloc_partials);
         if (e != cudaSuccess) {
            g_scratch_addr[dev] = nullptr;
            return noalloc_fail(LBM_ERR_CUDA, cudaGetErrorString(e));
         }
      }
      scratch = g_scratch_addr[dev];
   }

   GridDims g;
   g.nx = nx;
   g.ny = ny;
   g.nz = nz;
   g.ncell = ncell;
   g.plane = plane_stride;
   for (int d = 0; d < 3; d++) g.periodic[d] = periodic[d] ? 1 : 0;
   // runs of at least kNoAllocMinCells cells, a multiple of the block size,
   // in at most kNoAllocMaxBlocks blocks (2^28 / 4096 = 65536 cells at most)
   int64_t per_block = (ncell + kNoAllocMaxBlocks - 1) / kNoAllocMaxBlocks;
   per_block = per_block < kNoAllocMinCells ? kNoAllocMinCells : per_block;
   per_block = (per_block + kNoAllocThreads - 1) / kNoAllocThreads * kNoAllocThreads;
   const int nblocks = (int)((ncell + per_block - 1) / per_block);
   cudaStream_t st = static_cast<cudaStream_t>(stream);
   if (lattice == 19) {
      switch (storage) {
         case LBM_STORE_F64: e = launch_chunks<19, ST_F64>(g, dstrb, solid, readout, scratch, per_block, nblocks, st); break;
         case LBM_STORE_F32: e = launch_chunks<19, ST_F32>(g, dstrb, solid, readout, scratch, per_block, nblocks, st); break;
         case LBM_STORE_BF16: e = launch_chunks<19, ST_BF16>(g, dstrb, solid, readout, scratch, per_block, nblocks, st); break;
         default: e = launch_chunks<19, ST_F16>(g, dstrb, solid, readout, scratch, per_block, nblocks, st); break;
      }
   } else {
      switch (storage) {
         case LBM_STORE_F64: e = launch_chunks<27, ST_F64>(g, dstrb, solid, readout, scratch, per_block, nblocks, st); break;
         case LBM_STORE_F32: e = launch_chunks<27, ST_F32>(g, dstrb, solid, readout, scratch, per_block, nblocks, st); break;
         case LBM_STORE_BF16: e = launch_chunks<27, ST_BF16>(g, dstrb, solid, readout, scratch, per_block, nblocks, st); break;
         default: e = launch_chunks<27, ST_F16>(g, dstrb, solid, readout, scratch, per_block, nblocks, st); break;
      }
   }
   if (e != cudaSuccess) return noalloc_fail(LBM_ERR_CUDA, cudaGetErrorString(e));
   conserved_final_kernel<<<1, kReduceThreads, 0, st>>>(scratch, nblocks, out);
   e = cudaGetLastError();
   if (e != cudaSuccess) return noalloc_fail(LBM_ERR_CUDA, cudaGetErrorString(e));
   return LBM_OK;
}
