// C ABI implementation (include/lbm_gb300.h): handle lifetime, geometry,
// initialisation, the time loop and readouts.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/lbm_gb300.h"
#include "lbm_adjoint.cuh"
#include "lbm_aux.cuh"
#include "lbm_compact.cuh"
#include "lbm_dispatch.cuh"
#include "lbm_f64x.cuh"

using namespace lbm;

struct lbm_handle {
   lbm_config cfg;
   int Q = 19;
   int storage = ST_F64;
   int arith = AR_F64X;
   int elem = 8;
   int64_t ncell = 0, nfluid = 0, plane = 0, t = 0;
   uint64_t buffer_bytes = 0, device_bytes = 0;
   void* buf[2] = {nullptr, nullptr};
   int cur = 0;                    // AB: buffer holding the latest state
   uint32_t* links = nullptr;      // null when the box is fully periodic and has no solids
   uint8_t* solid_dev = nullptr;   // scratch for building links
   double* force_field = nullptr;  // planar [3][plane]
   float* force_field_f = nullptr;
   double* porosity = nullptr;
   float* porosity_f = nullptr;
   double* staging = nullptr;      // one dense double plane (at least kMinStaging doubles)
   size_t staging_elems = 0;
   cudaStream_t copy_stream = nullptr;   // host <-> staging copies of the chunked transfers
   cudaEvent_t chunk_ready[2] = {nullptr, nullptr};
   cudaEvent_t chunk_free[2] = {nullptr, nullptr};
   double* partials = nullptr;     // reduction scratch: plane partials or 4 doubles per loss block
   double* reduce_out = nullptr;   // 4 doubles
   uint32_t* sched = nullptr;      // tile counter of the persistent step kernels (zero between launches)
   cudaStream_t stream = nullptr;
   // Compact fluid-only storage (cfg.compact): the steps run on cbuf; buf[0]
   // is the dense copy that set-up, readouts and host transfers use, brought
   // up to date (expand / compress) when the other copy was written last.
   bool compact = false;
   void* cbuf = nullptr;
   uint64_t cbuf_bytes = 0;
   uint32_t nf32 = 0, cplane = 0, nrow_tiles = 0;
   uint32_t* dcell = nullptr;       // [nf] dense cell of each fluid cell
   OddTile* ctiles = nullptr;       // [nrow_tiles] row tiles of the odd step
   uint2* cu = nullptr;             // [nrow_tiles * 32] row counts of the tile lanes
   uint32_t* clk = nullptr;         // [nrow_tiles * 32] link words of the tile lanes
   size_t compact_meta_bytes[4] = {0, 0, 0, 0};
   bool dense_current = true;       // buf[0] holds the latest state
   bool compact_current = false;    // cbuf holds the latest state
   std::string err;
};

namespace {

constexpr int kReduceBlocks = 152 * 8;
constexpr size_t kMinStaging = 1 << 16;   // doubles

lbm_status fail(lbm_handle* h, lbm_status s, const char* fmt, ...)
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

lbm_status cuda_fail(lbm_handle* h, cudaError_t e, const char* what)
{
   return fail(h, LBM_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

#define LBM_CUDA(h, call)                                            \
   do {                                                              \
      cudaError_t e_ = (call);                                       \
      if (e_ != cudaSuccess) return cuda_fail((h), e_, #call);       \
   } while (0)

GridDims dims_of(const lbm_handle* h)
{
   GridDims g;
   g.nx = h->cfg.nx;
   g.ny = h->cfg.ny;
   g.nz = h->cfg.nz;
   g.ncell = h->ncell;
   g.plane = h->plane;
   for (int d = 0; d < 3; d++) g.periodic[d] = h->cfg.periodic[d] ? 1 : 0;
   return g;
}

unsigned blocks_for(int64_t n, int threads) { return (unsigned)((n + threads - 1) / threads); }

bool fully_periodic(const lbm_handle* h)
{
   return h->cfg.periodic[0] && h->cfg.periodic[1] && h->cfg.periodic[2];
}

lbm_status dev_alloc(lbm_handle* h, void** p, size_t bytes)
{
   if (h->cfg.max_device_bytes && h->device_bytes + bytes > h->cfg.max_device_bytes)
      return fail(h, LBM_ERR_OUT_OF_MEMORY, "device allocation of %zu bytes exceeds max_device_bytes=%llu",
                  bytes, (unsigned long long)h->cfg.max_device_bytes);
   cudaError_t e = cudaMalloc(p, bytes);
   if (e != cudaSuccess) {
      cudaGetLastError();
      *p = nullptr;
      return fail(h, LBM_ERR_OUT_OF_MEMORY, "cudaMalloc(%zu): %s", bytes, cudaGetErrorString(e));
   }
   h->device_bytes += bytes;
   return LBM_OK;
}

void dev_free(lbm_handle* h, void* p, size_t bytes)
{
   if (!p) return;
   cudaFree(p);
   h->device_bytes -= std::min<uint64_t>(h->device_bytes, bytes);
}

// Step-kernel parameters for the cell range [start, end).
KParams make_params(const lbm_handle* h, int64_t start, int64_t end, Launch& L)
{
   KParams p;
   std::memset(&p, 0, sizeof(p));
   const lbm_config& c = h->cfg;
   p.nx = c.nx;
   p.ny = c.ny;
   p.nz = c.nz;
   p.ncell = h->ncell;
   p.plane = h->plane;
   p.cstart = start;
   p.cend = end;
   const int64_t nxy = (int64_t)c.nx * c.ny;
   const int64_t z0 = start / nxy, z1 = (end - 1) / nxy + 1;
   p.z0 = (int)z0;
   set_collision_constants(p, h->Q, c.omega, c.force,
                           (c.unroll && h->Q == 19 && c.prop_pattern == LBM_PATTERN_AA) ? 1 : 0);
   p.links = h->links;
   p.force_field = h->force_field;
   p.force_field_f = h->force_field_f;
   p.porosity = h->porosity;
   p.porosity_f = h->porosity_f;
   p.sched = h->sched;
   int bx = (int)std::min<int64_t>(256, ((c.nx + 31) / 32) * 32);
   L.block = dim3(bx, 1, 1);
   L.grid = dim3((c.nx + bx - 1) / bx, c.ny, (unsigned)(z1 - z0));
   L.stream = h->stream;
   L.idx32 = (uint64_t)h->plane * (uint64_t)h->elem < (1ull << 32);   // plane stride in bytes
   L.pair = h->storage != ST_F64 && c.nx % 2 == 0 && start == 0 && end == h->ncell;
   const int half = c.nx / 2;
   const int pbx = (int)std::min<int64_t>(256, ((half + 31) / 32) * 32);
   L.pair_block = dim3(pbx, 1, 1);
   L.pair_grid = dim3((half + pbx - 1) / pbx, c.ny, (unsigned)(z1 - z0));
   L.async = h->storage == ST_F64 && h->arith == AR_F64X && start == 0 && end == h->ncell && L.idx32;
   L.async_low = h->storage != ST_F64 && start == 0 && end == h->ncell && (uint64_t)h->Q * (uint64_t)h->plane < (1ull << 32);
   L.ag = async_geom(c.nx, c.ny, c.nz);
   return p;
}

lbm_status launch(lbm_handle* h, int kind, const void* src, void* dst, int64_t start, int64_t count)
{
   if (count <= 0) return LBM_OK;
   Launch L;
   const KParams p = make_params(h, start, start + count, L);
   const bool links = h->links != nullptr;
   const bool fields = h->force_field || h->force_field_f || h->porosity || h->porosity_f;
   cudaError_t e;
   if (h->Q == 19) {
      e = h->storage == ST_F64 ? launch_step_q19_f64(h->arith, kind, L, p, src, dst, links, fields)
                               : launch_step_q19_low(h->storage, kind, L, p, src, dst, links, fields);
   } else {
      e = h->storage == ST_F64 ? launch_step_q27_f64(h->arith, kind, L, p, src, dst, links, fields)
                               : launch_step_q27_low(h->storage, kind, L, p, src, dst, links, fields);
   }
   if (e != cudaSuccess) return cuda_fail(h, e, "step kernel launch");
   return LBM_OK;
}

template <template <int, int> class F, typename... A>
void dispatch_q_st(int Q, int st, A&&... a)
{
   if (Q == 19) {
      switch (st) {
         case ST_F64: F<19, ST_F64>::run(a...); break;
         case ST_F32: F<19, ST_F32>::run(a...); break;
         case ST_BF16: F<19, ST_BF16>::run(a...); break;
         default: F<19, ST_F16>::run(a...); break;
      }
   } else {
      switch (st) {
         case ST_F64: F<27, ST_F64>::run(a...); break;
         case ST_F32: F<27, ST_F32>::run(a...); break;
         case ST_BF16: F<27, ST_BF16>::run(a...); break;
         default: F<27, ST_F16>::run(a...); break;
      }
   }
}

template <int Q, int ST>
struct InitEq {
   static void run(const lbm_handle* h, int64_t c0, int64_t count, const double* rho, const double* u,
                   int64_t in_stride, int aa)
   {
      init_eq_kernel<Q, ST><<<blocks_for(count, 256), 256, 0, h->stream>>>(dims_of(h), c0, count, rho, u, in_stride,
                                                                            h->buf[0], h->buf[1], aa);
   }
};

template <int Q, int ST>
struct ImportPlane {
   static void run(const lbm_handle* h, int slot, double w, void* b0, void* b1)
   {
      import_plane_kernel<ST><<<blocks_for(h->ncell, 256), 256, 0, h->stream>>>(dims_of(h), h->staging, slot, w,
                                                                                 b0, b1);
   }
};

template <int Q, int ST>
struct ExportPlane {
   static void run(const lbm_handle* h, const void* buf, int s, int mode)
   {
      export_plane_kernel<Q, ST><<<blocks_for(h->ncell, 256), 256, 0, h->stream>>>(dims_of(h), buf, h->links,
                                                                                    plane_dir(Q, s), mode,
                                                                                    h->staging);
   }
};

template <int Q, int ST>
struct Macros {
   static void run(const lbm_handle* h, int64_t c0, int64_t count, const void* buf, int mode, double* rho,
                   double* u, int64_t out_stride)
   {
      macros_kernel<Q, ST><<<blocks_for(count, 256), 256, 0, h->stream>>>(dims_of(h), c0, count, buf, h->links,
                                                                           mode, rho, u, out_stride);
   }
};

template <int Q, int ST>
struct Conserved {
   static void run(const lbm_handle* h, const void* buf, int mode, double* partials, double* out)
   {
      PlanePartial* part = reinterpret_cast<PlanePartial*>(partials);
      const int64_t per_range = plane_per_range(h->ncell);
      const int nblocks = plane_blocks(Q, h->ncell);
      conserved_plane_kernel<Q, ST><<<nblocks, kReduceThreads, 0, h->stream>>>(dims_of(h), buf, h->links, mode,
                                                                              per_range, part);
      conserved_plane_final_kernel<Q><<<1, kReduceThreads, 0, h->stream>>>(part, nblocks, mode, out);
   }
};

double weight(int Q, int s)
{
   const int n2 = lat_norm2(Q, s);
   if (Q == 19) return n2 == 0 ? 1.0 / 3.0 : (n2 == 1 ? 1.0 / 18.0 : 1.0 / 36.0);
   return n2 == 0 ? 8.0 / 27.0 : (n2 == 1 ? 2.0 / 27.0 : (n2 == 2 ? 1.0 / 54.0 : 1.0 / 216.0));
}

// Buffer the reference reads back, and how its slots map to directions.
const void* readout_buffer(const lbm_handle* h)
{
   return h->cfg.prop_pattern == LBM_PATTERN_AA ? h->buf[0] : h->buf[h->cur];
}

// Export mode for logical populations: 0 stored slot s, 1 own slot opp(s),
// 2 pull gather.
int logical_mode(const lbm_handle* h)
{
   if (h->cfg.prop_pattern == LBM_PATTERN_AA) return (h->t % 2 == 0) ? 1 : 2;
   return h->cfg.pull ? 2 : 0;
}

lbm_status check_handle(const lbm_handle* h) { return h ? LBM_OK : LBM_ERR_INVALID_ARGUMENT; }

// Compact storage: make the dense copy current before it is read.
lbm_status dense_for_read(lbm_handle* h)
{
   if (!h->compact || h->dense_current) return LBM_OK;
   cudaError_t e = launch_compact_expand(h->Q, h->storage, h->dcell, h->nf32, h->cplane, h->cbuf, h->buf[0],
                                         h->plane, h->stream);
   if (e != cudaSuccess) return cuda_fail(h, e, "compact expand");
   h->dense_current = true;
   return LBM_OK;
}

// Compact storage: the dense copy was written; the compact one is stale.
void dense_written(lbm_handle* h)
{
   h->dense_current = true;
   h->compact_current = false;
}

CompactGeom compact_geom(const lbm_handle* h)
{
   CompactGeom g;
   g.tiles = h->ctiles;
   g.u = h->cu;
   g.lk = h->clk;
   g.nrow_tiles = h->nrow_tiles;
   g.nf = h->nf32;
   g.cplane = h->cplane;
   for (int k = 0; k < 27; k++) g.soff[k] = (uint32_t)k * h->cplane;
   return g;
}

void free_compact(lbm_handle* h)
{
   void* ptrs[4] = {h->dcell, h->ctiles, h->cu, h->clk};
   for (int k = 0; k < 4; k++) {
      dev_free(h, ptrs[k], h->compact_meta_bytes[k]);
      h->compact_meta_bytes[k] = 0;
   }
   h->dcell = h->clk = nullptr;
   h->ctiles = nullptr;
   h->cu = nullptr;
   dev_free(h, h->cbuf, h->cbuf_bytes);
   h->cbuf = nullptr;
   h->cbuf_bytes = 0;
}

// The compact numbering of the fluid cells (dense order, solids left out),
// the row tiles of the odd step with their lanes' row counts, and the compact
// buffer, from the host mask (null: every cell fluid); the lanes' link words
// are gathered from the dense ones.
lbm_status build_compact(lbm_handle* h, const uint8_t* solid)
{
   const int nx = h->cfg.nx;
   std::vector<uint32_t> dcell, ucounts;
   std::vector<OddTile> tiles;
   build_row_tiles(nx, h->cfg.ny, h->cfg.nz, solid, dcell, tiles, ucounts);
   free_compact(h);
   h->nf32 = (uint32_t)dcell.size();
   h->cplane = (h->nf32 + 255u) / 256u * 256u;
   if ((uint64_t)h->Q * h->cplane >= (1ull << 32) || tiles.size() >= (1u << 27))
      return fail(h, LBM_ERR_UNSUPPORTED, "compact storage needs Q * fluid cells below 2^32");
   h->nrow_tiles = (uint32_t)tiles.size();
   struct Part {
      void** dst;
      const void* src;
      size_t bytes;
   } parts[4] = {{(void**)&h->dcell, dcell.data(), 4 * dcell.size()},
                 {(void**)&h->ctiles, tiles.data(), sizeof(OddTile) * tiles.size()},
                 {(void**)&h->cu, ucounts.data(), sizeof(uint32_t) * ucounts.size()},
                 {(void**)&h->clk, nullptr, 2 * ucounts.size()}};
   for (int k = 0; k < 4; k++) {
      const size_t bytes = std::max<size_t>(parts[k].bytes, 16);
      lbm_status st = dev_alloc(h, parts[k].dst, bytes);
      if (st != LBM_OK) return st;
      h->compact_meta_bytes[k] = bytes;
      if (parts[k].src && parts[k].bytes)
         LBM_CUDA(h, cudaMemcpyAsync(*parts[k].dst, parts[k].src, parts[k].bytes, cudaMemcpyHostToDevice, h->stream));
   }
   LBM_CUDA(h, launch_compact_links(h->ctiles, h->nrow_tiles, h->dcell, h->links, nx, h->clk, h->stream));
   h->cbuf_bytes = std::max<uint64_t>((uint64_t)h->cplane * h->Q * h->elem, 16);
   lbm_status st = dev_alloc(h, &h->cbuf, h->cbuf_bytes);
   if (st != LBM_OK) return st;
   // the plane padding past nf holds zeros (the even step's tail pair runs on it)
   LBM_CUDA(h, cudaMemsetAsync(h->cbuf, 0, h->cbuf_bytes, h->stream));
   // the host vectors go out of scope: wait for the copies
   LBM_CUDA(h, cudaStreamSynchronize(h->stream));
   h->compact_current = false;
   return LBM_OK;
}

}  // namespace

extern "C" {

const char* lbm_status_string(lbm_status s)
{
   switch (s) {
      case LBM_OK: return "ok";
      case LBM_ERR_INVALID_ARGUMENT: return "invalid argument";
      case LBM_ERR_OUT_OF_MEMORY: return "out of device memory";
      case LBM_ERR_CUDA: return "CUDA error";
      case LBM_ERR_DIVERGED: return "diverged (non-finite conserved sums)";
      case LBM_ERR_UNSUPPORTED: return "unsupported";
      case LBM_ERR_STATE: return "invalid state";
   }
   return "unknown status";
}

const char* lbm_last_error(const lbm_handle* h)
{
   if (!h) return "null handle";
   return h->err.c_str();
}

lbm_status lbm_config_default(lbm_config* cfg)
{
   if (!cfg) return LBM_ERR_INVALID_ARGUMENT;
   std::memset(cfg, 0, sizeof(*cfg));
   cfg->lattice = 19;
   cfg->prop_pattern = LBM_PATTERN_AA;
   cfg->nx = cfg->ny = cfg->nz = 16;
   cfg->periodic[0] = cfg->periodic[1] = cfg->periodic[2] = 1;
   cfg->omega = 1.0;
   cfg->force[0] = 0.000001;
   cfg->storage = LBM_STORE_F64;
   cfg->arithmetic = LBM_ARITH_AUTO;
   return LBM_OK;
}

void lbm_destroy(lbm_handle* h)
{
   if (!h) return;
   int prev = -1;
   cudaGetDevice(&prev);
   cudaSetDevice(h->cfg.device);
   if (h->stream) cudaStreamSynchronize(h->stream);
   cudaFree(h->buf[0]);
   cudaFree(h->buf[1]);
   cudaFree(h->links);
   cudaFree(h->solid_dev);
   cudaFree(h->force_field);
   cudaFree(h->force_field_f);
   cudaFree(h->porosity);
   cudaFree(h->porosity_f);
   cudaFree(h->staging);
   if (h->copy_stream) {
      cudaStreamSynchronize(h->copy_stream);
      cudaStreamDestroy(h->copy_stream);
   }
   for (int k = 0; k < 2; k++) {
      if (h->chunk_ready[k]) cudaEventDestroy(h->chunk_ready[k]);
      if (h->chunk_free[k]) cudaEventDestroy(h->chunk_free[k]);
   }
   cudaFree(h->partials);
   cudaFree(h->reduce_out);
   cudaFree(h->sched);
   cudaFree(h->cbuf);
   cudaFree(h->dcell);
   cudaFree(h->ctiles);
   cudaFree(h->cu);
   cudaFree(h->clk);
   if (prev >= 0) cudaSetDevice(prev);
   delete h;
}

lbm_status lbm_create(const lbm_config* cfg, lbm_handle** out)
{
   if (!cfg || !out) return LBM_ERR_INVALID_ARGUMENT;
   *out = nullptr;
   lbm_handle* h = new (std::nothrow) lbm_handle;
   if (!h) return LBM_ERR_OUT_OF_MEMORY;
   h->cfg = *cfg;
   lbm_status st = LBM_OK;
   const lbm_config& c = *cfg;
   const int64_t ncell = (int64_t)c.nx * c.ny * c.nz;
   if (c.lattice != 19 && c.lattice != 27) st = fail(h, LBM_ERR_INVALID_ARGUMENT, "lattice must be 19 or 27");
   else if (c.nx < 1 || c.ny < 1 || c.nz < 1 || c.ny > 65535 || c.nz > 65535)
      st = fail(h, LBM_ERR_INVALID_ARGUMENT, "grid dimensions out of range (ny, nz <= 65535)");
   else if (ncell > (int64_t)INT32_MAX)
      st = fail(h, LBM_ERR_INVALID_ARGUMENT, "nx*ny*nz must be below 2^31 cells");
   else if (c.prop_pattern != LBM_PATTERN_AA && c.prop_pattern != LBM_PATTERN_AB)
      st = fail(h, LBM_ERR_INVALID_ARGUMENT, "prop_pattern must be 0 (AB) or 1 (AA)");
   else if (c.storage < LBM_STORE_F64 || c.storage > LBM_STORE_F16)
      st = fail(h, LBM_ERR_INVALID_ARGUMENT, "unknown storage");
   else if (!(c.omega > 0.0 && c.omega < 2.0))
      st = fail(h, LBM_ERR_INVALID_ARGUMENT, "omega must lie in (0, 2)");
   else if (c.arithmetic < LBM_ARITH_AUTO || c.arithmetic > LBM_ARITH_F32)
      st = fail(h, LBM_ERR_INVALID_ARGUMENT, "unknown arithmetic");
   else if (c.compact != 0 && c.compact != 1)
      st = fail(h, LBM_ERR_INVALID_ARGUMENT, "compact must be 0 or 1");
   else if (c.compact && (c.prop_pattern != LBM_PATTERN_AA || c.storage == LBM_STORE_F64))
      st = fail(h, LBM_ERR_UNSUPPORTED, "compact storage runs AA steps with F32, BF16 or F16 storage");
   else if (c.compact && c.nx > 65535)
      st = fail(h, LBM_ERR_UNSUPPORTED, "compact storage needs nx <= 65535");
   if (st == LBM_OK) {
      h->Q = c.lattice;
      h->storage = c.storage;
      if (c.storage == LBM_STORE_F64) {
         h->arith = (c.arithmetic == LBM_ARITH_F64) ? AR_F64 : AR_F64X;
         if (c.arithmetic == LBM_ARITH_F32)
            st = fail(h, LBM_ERR_UNSUPPORTED, "FP64 storage computes in F64 or F64X arithmetic");
      } else {
         h->arith = AR_F32;
         if (c.arithmetic == LBM_ARITH_F64 || c.arithmetic == LBM_ARITH_F64X)
            st = fail(h, LBM_ERR_UNSUPPORTED, "shifted FP32/BF16/FP16 storage computes in FP32");
      }
      h->elem = c.storage == LBM_STORE_F64 ? 8 : (c.storage == LBM_STORE_F32 ? 4 : 2);
      h->compact = c.compact != 0;
      h->ncell = ncell;
      h->nfluid = ncell;
      // Planes start on 512-byte boundaries.
      const int64_t align = 512 / h->elem;
      h->plane = (ncell + align - 1) / align * align;
      h->buffer_bytes = (uint64_t)h->plane * h->Q * h->elem;
   }
   if (st == LBM_OK) {
      int ndev = 0;
      cudaError_t e = cudaGetDeviceCount(&ndev);
      if (e != cudaSuccess || c.device < 0 || c.device >= ndev)
         st = fail(h, LBM_ERR_CUDA, "no CUDA device %d (%s)", c.device, cudaGetErrorString(e));
      else if ((e = cudaSetDevice(c.device)) != cudaSuccess)
         st = cuda_fail(h, e, "cudaSetDevice");
   }
   if (st == LBM_OK) st = dev_alloc(h, &h->buf[0], h->buffer_bytes);
   if (st == LBM_OK && c.prop_pattern == LBM_PATTERN_AB) st = dev_alloc(h, &h->buf[1], h->buffer_bytes);
   h->staging_elems = std::max<size_t>((size_t)h->ncell, kMinStaging);
   if (st == LBM_OK) st = dev_alloc(h, (void**)&h->staging, sizeof(double) * h->staging_elems);
   if (st == LBM_OK) {
      // the plane reduction's partials, or the loss reduction's 4 doubles per block
      const size_t plane_bytes = sizeof(PlanePartial) * (size_t)27 * kPlaneRanges;
      const size_t loss_bytes = sizeof(double) * 4 * kReduceBlocks;
      st = dev_alloc(h, (void**)&h->partials, plane_bytes > loss_bytes ? plane_bytes : loss_bytes);
   }
   if (st == LBM_OK) st = dev_alloc(h, (void**)&h->reduce_out, sizeof(double) * 4);
   if (st == LBM_OK) st = dev_alloc(h, (void**)&h->sched, 4 * kFeedWords);
   if (st == LBM_OK) {
      const cudaError_t e = cudaMemset(h->sched, 0, 4 * kFeedWords);
      if (e != cudaSuccess) st = cuda_fail(h, e, "cudaMemset");
   }
   if (st == LBM_OK) st = lbm_set_solid(h, nullptr);
   if (st == LBM_OK) st = lbm_init_equilibrium(h, nullptr, nullptr);
   if (st != LBM_OK) {
      std::string msg = h->err;
      lbm_destroy(h);
      fprintf(stderr, "lbm_create: %s\n", msg.c_str());
      return st;
   }
   *out = h;
   return LBM_OK;
}

lbm_status lbm_get_info(const lbm_handle* h, lbm_info* info)
{
   if (!h || !info) return LBM_ERR_INVALID_ARGUMENT;
   info->ncell = h->ncell;
   info->nfluid = h->nfluid;
   info->time_step = h->t;
   info->plane_stride = h->plane;
   info->buffer_bytes = h->buffer_bytes;
   info->device_bytes = h->device_bytes;
   info->bytes_per_update = 2 * h->Q * h->elem;
   info->lattice = h->Q;
   info->storage = h->storage;
   info->arithmetic = h->arith == AR_F64 ? LBM_ARITH_F64 : (h->arith == AR_F64X ? LBM_ARITH_F64X : LBM_ARITH_F32);
   return LBM_OK;
}

lbm_status lbm_set_stream(lbm_handle* h, void* stream)
{
   if (!h) return LBM_ERR_INVALID_ARGUMENT;
   h->stream = static_cast<cudaStream_t>(stream);
   return LBM_OK;
}

lbm_status lbm_synchronize(lbm_handle* h)
{
   if (!h) return LBM_ERR_INVALID_ARGUMENT;
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   LBM_CUDA(h, cudaStreamSynchronize(h->stream));
   return LBM_OK;
}

lbm_status lbm_set_solid(lbm_handle* h, const uint8_t* solid)
{
   if (!h) return LBM_ERR_INVALID_ARGUMENT;
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   // the state carries over in the dense copy
   lbm_status st0 = dense_for_read(h);
   if (st0 != LBM_OK) return st0;
   int64_t nsolid = 0;
   if (solid)
      for (int64_t c = 0; c < h->ncell; c++) nsolid += solid[c] ? 1 : 0;
   h->nfluid = h->ncell - nsolid;
   const bool need_links = nsolid > 0 || !fully_periodic(h);
   if (!need_links) {
      dev_free(h, h->links, sizeof(uint32_t) * (size_t)h->ncell);
      h->links = nullptr;
      if (h->compact) return build_compact(h, solid);
      return LBM_OK;
   }
   if (!h->links) {
      lbm_status st = dev_alloc(h, (void**)&h->links, sizeof(uint32_t) * (size_t)h->ncell);
      if (st != LBM_OK) return st;
   }
   uint8_t* sd = nullptr;
   if (solid) {
      lbm_status st = dev_alloc(h, (void**)&sd, (size_t)h->ncell);
      if (st != LBM_OK) return st;
      LBM_CUDA(h, cudaMemcpyAsync(sd, solid, (size_t)h->ncell, cudaMemcpyHostToDevice, h->stream));
   }
   const GridDims g = dims_of(h);
   if (h->Q == 19) build_links_kernel<19><<<blocks_for(h->ncell, 256), 256, 0, h->stream>>>(g, sd, h->links);
   else build_links_kernel<27><<<blocks_for(h->ncell, 256), 256, 0, h->stream>>>(g, sd, h->links);
   LBM_CUDA(h, cudaGetLastError());
   LBM_CUDA(h, cudaStreamSynchronize(h->stream));
   dev_free(h, sd, (size_t)h->ncell);
   if (h->compact) return build_compact(h, solid);
   return LBM_OK;
}

lbm_status lbm_geometry_cylinder(double simulation_size, int dims[3], uint8_t* solid)
{
   // src/geometries/Geometry.cpp:59-71 (lengths) and :112-140 (mask): radius
   // and axial length truncated to int; a cell is fluid when
   // int(distance to the axis) <= radius, the axis at radius + 1.5.
   if (!dims || !(simulation_size > 0.0)) return LBM_ERR_INVALID_ARGUMENT;
   const int radius = (int)(8.0 * simulation_size);
   const int axial = (int)(84.0 * simulation_size);
   if (radius < 1 || axial < 1) return LBM_ERR_INVALID_ARGUMENT;
   dims[0] = axial;
   dims[1] = 2 * radius + 3;
   dims[2] = 2 * radius + 3;
   if (!solid) return LBM_OK;
   const double r = (double)((dims[1] - 3) / 2);
   const double axis = r + 1.5;
   for (int k = 0; k < dims[2]; k++)
      for (int j = 0; j < dims[1]; j++) {
         const int dist = (int)std::sqrt(std::pow(j - axis, 2.0) + std::pow(k - axis, 2.0));
         const uint8_t s = dist <= r ? 0 : 1;
         for (int i = 0; i < dims[0]; i++) solid[(size_t)i + (size_t)dims[0] * ((size_t)j + (size_t)dims[1] * k)] = s;
      }
   return LBM_OK;
}

static lbm_status set_field(lbm_handle* h, const double* host, int ncomp, double** d64, float** d32)
{
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   const size_t n = (size_t)h->plane * ncomp;
   if (!host) {
      dev_free(h, *d64, sizeof(double) * n);
      dev_free(h, *d32, sizeof(float) * n);
      *d64 = nullptr;
      *d32 = nullptr;
      return LBM_OK;
   }
   if (h->storage == ST_F64) {
      if (!*d64) {
         lbm_status st = dev_alloc(h, (void**)d64, sizeof(double) * n);
         if (st != LBM_OK) return st;
      }
      for (int k = 0; k < ncomp; k++)
         LBM_CUDA(h, cudaMemcpyAsync(*d64 + (size_t)k * h->plane, host + (size_t)k * h->ncell,
                                     sizeof(double) * (size_t)h->ncell, cudaMemcpyHostToDevice, h->stream));
   } else {
      if (!*d32) {
         lbm_status st = dev_alloc(h, (void**)d32, sizeof(float) * n);
         if (st != LBM_OK) return st;
      }
      std::vector<float> tmp((size_t)h->ncell);
      for (int k = 0; k < ncomp; k++) {
         for (int64_t c = 0; c < h->ncell; c++) tmp[(size_t)c] = (float)host[(size_t)k * h->ncell + c];
         LBM_CUDA(h, cudaMemcpy(*d32 + (size_t)k * h->plane, tmp.data(), sizeof(float) * (size_t)h->ncell,
                                cudaMemcpyHostToDevice));
      }
   }
   LBM_CUDA(h, cudaStreamSynchronize(h->stream));
   return LBM_OK;
}

lbm_status lbm_set_force_field(lbm_handle* h, const double* field)
{
   if (!h) return LBM_ERR_INVALID_ARGUMENT;
   if (h->compact && field) return fail(h, LBM_ERR_UNSUPPORTED, "compact storage has no per-cell fields");
   return set_field(h, field, 3, &h->force_field, &h->force_field_f);
}

lbm_status lbm_set_porosity(lbm_handle* h, const double* porosity)
{
   if (!h) return LBM_ERR_INVALID_ARGUMENT;
   if (h->compact && porosity) return fail(h, LBM_ERR_UNSUPPORTED, "compact storage has no per-cell fields");
   if (porosity)
      for (int64_t c = 0; c < h->ncell; c++)
         if (!(porosity[c] >= 0.0 && porosity[c] <= 1.0))
            return fail(h, LBM_ERR_INVALID_ARGUMENT, "porosity[%lld] = %g outside [0, 1]", (long long)c,
                        porosity[c]);
   return set_field(h, porosity, 1, &h->porosity, &h->porosity_f);
}

// Copy stream and events of the chunked host transfers, made on first use.
static lbm_status ensure_copy_stream(lbm_handle* h)
{
   if (h->copy_stream) return LBM_OK;
   LBM_CUDA(h, cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
   for (int k = 0; k < 2; k++) {
      LBM_CUDA(h, cudaEventCreateWithFlags(&h->chunk_ready[k], cudaEventDisableTiming));
      LBM_CUDA(h, cudaEventCreateWithFlags(&h->chunk_free[k], cudaEventDisableTiming));
   }
   return LBM_OK;
}

// Host arrays move through the two halves of the staging plane in chunks of
// cells: while the kernel works on one half, the copy stream fills (or
// drains) the other.  ncomp planar components of `chunk` cells fit one half.
static int64_t chunk_cells(const lbm_handle* h, int ncomp)
{
   return (int64_t)((h->staging_elems / 2) / (size_t)ncomp);
}

lbm_status lbm_init_equilibrium(lbm_handle* h, const double* rho, const double* u)
{
   if (!h) return LBM_ERR_INVALID_ARGUMENT;
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   const int aa = h->cfg.prop_pattern == LBM_PATTERN_AA ? 1 : 0;
   const int64_t n = h->ncell;
   if (!rho && !u) {
      dispatch_q_st<InitEq>(h->Q, h->storage, h, (int64_t)0, n, (const double*)nullptr, (const double*)nullptr,
                            n, aa);
      LBM_CUDA(h, cudaGetLastError());
   } else {
      lbm_status st = ensure_copy_stream(h);
      if (st != LBM_OK) return st;
      const int ncomp = (rho ? 1 : 0) + (u ? 3 : 0);
      const int64_t chunk = chunk_cells(h, ncomp);
      const size_t half = h->staging_elems / 2;
      // staging is free once the work already queued on the handle's stream is done
      for (int b = 0; b < 2; b++) LBM_CUDA(h, cudaEventRecord(h->chunk_free[b], h->stream));
      for (int64_t c0 = 0, k = 0; c0 < n; c0 += chunk, k++) {
         const int64_t cnt = std::min<int64_t>(chunk, n - c0);
         const int b = (int)(k & 1);
         double* dst = h->staging + b * half;
         LBM_CUDA(h, cudaStreamWaitEvent(h->copy_stream, h->chunk_free[b], 0));
         double* drho = nullptr;
         double* du = nullptr;
         if (rho) {
            drho = dst;
            LBM_CUDA(h, cudaMemcpyAsync(drho, rho + c0, sizeof(double) * cnt, cudaMemcpyHostToDevice,
                                        h->copy_stream));
         }
         if (u) {
            du = dst + (rho ? cnt : 0);
            for (int d = 0; d < 3; d++)
               LBM_CUDA(h, cudaMemcpyAsync(du + d * cnt, u + (size_t)d * n + c0, sizeof(double) * cnt,
                                           cudaMemcpyHostToDevice, h->copy_stream));
         }
         LBM_CUDA(h, cudaEventRecord(h->chunk_ready[b], h->copy_stream));
         LBM_CUDA(h, cudaStreamWaitEvent(h->stream, h->chunk_ready[b], 0));
         dispatch_q_st<InitEq>(h->Q, h->storage, h, c0, cnt, (const double*)drho, (const double*)du, cnt, aa);
         LBM_CUDA(h, cudaGetLastError());
         LBM_CUDA(h, cudaEventRecord(h->chunk_free[b], h->stream));
      }
   }
   cudaError_t e = cudaStreamSynchronize(h->stream);
   if (e != cudaSuccess) return cuda_fail(h, e, "init_eq sync");
   h->t = 0;
   h->cur = 0;
   dense_written(h);
   return LBM_OK;
}

lbm_status lbm_set_populations(lbm_handle* h, const double* f, int layout)
{
   if (!h || !f || (layout != LBM_LAYOUT_RAW && layout != LBM_LAYOUT_LOGICAL)) return LBM_ERR_INVALID_ARGUMENT;
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   const bool aa = h->cfg.prop_pattern == LBM_PATTERN_AA;
   if (layout == LBM_LAYOUT_LOGICAL) {
      h->t = 0;
      h->cur = 0;
   }
   for (int s = 0; s < h->Q; s++) {
      LBM_CUDA(h, cudaMemcpyAsync(h->staging, f + (size_t)s * h->ncell, sizeof(double) * (size_t)h->ncell,
                                  cudaMemcpyHostToDevice, h->stream));
      int slot = s;
      void* b0 = aa ? h->buf[0] : h->buf[h->cur];
      void* b1 = nullptr;
      if (layout == LBM_LAYOUT_LOGICAL) {
         if (aa) slot = lat_opp(h->Q, s);
         else b1 = h->buf[1 - h->cur];
      }
      dispatch_q_st<ImportPlane>(h->Q, h->storage, h, slot, weight(h->Q, s), b0, b1);
      LBM_CUDA(h, cudaGetLastError());
   }
   LBM_CUDA(h, cudaStreamSynchronize(h->stream));
   dense_written(h);
   return LBM_OK;
}

lbm_status lbm_get_populations(lbm_handle* h, double* f, int layout)
{
   if (!h || !f || (layout != LBM_LAYOUT_RAW && layout != LBM_LAYOUT_LOGICAL)) return LBM_ERR_INVALID_ARGUMENT;
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   lbm_status st = dense_for_read(h);
   if (st != LBM_OK) return st;
   const int mode = layout == LBM_LAYOUT_RAW ? 0 : logical_mode(h);
   const void* buf = readout_buffer(h);
   for (int s = 0; s < h->Q; s++) {
      dispatch_q_st<ExportPlane>(h->Q, h->storage, h, buf, s, mode);
      LBM_CUDA(h, cudaGetLastError());
      LBM_CUDA(h, cudaMemcpyAsync(f + (size_t)s * h->ncell, h->staging, sizeof(double) * (size_t)h->ncell,
                                  cudaMemcpyDeviceToHost, h->stream));
   }
   LBM_CUDA(h, cudaStreamSynchronize(h->stream));
   return LBM_OK;
}

// AA steps on the compact buffer.
static lbm_status step_compact(lbm_handle* h, int nsteps)
{
   if (nsteps == 0) return LBM_OK;
   if (!h->compact_current) {
      LBM_CUDA(h, launch_compact_compress(h->Q, h->storage, h->dcell, h->nf32, h->cplane, h->buf[0], h->plane,
                                          h->cbuf, h->stream));
      h->compact_current = true;
   }
   h->dense_current = false;
   Launch L;
   const KParams p = make_params(h, 0, h->ncell, L);
   const CompactGeom g = compact_geom(h);
   for (int i = 0; i < nsteps; i++) {
      const int kind = (h->t % 2 == 0) ? K_AA_EVEN : K_AA_ODD;
      cudaError_t e = launch_compact_step(h->Q, h->storage, kind, p, g, h->cbuf, h->stream);
      if (e != cudaSuccess) return cuda_fail(h, e, "compact step kernel launch");
      h->t++;
   }
   return LBM_OK;
}

lbm_status lbm_step(lbm_handle* h, int nsteps)
{
   if (!h || nsteps < 0) return LBM_ERR_INVALID_ARGUMENT;
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   if (h->compact) return step_compact(h, nsteps);
   for (int i = 0; i < nsteps; i++) {
      lbm_status st;
      if (h->cfg.prop_pattern == LBM_PATTERN_AA) {
         const int kind = (h->t % 2 == 0) ? K_AA_EVEN : K_AA_ODD;
         st = launch(h, kind, h->buf[0], h->buf[0], 0, h->ncell);
      } else {
         const int kind = h->cfg.pull ? K_AB_PULL : K_AB_PUSH;
         st = launch(h, kind, h->buf[h->cur], h->buf[1 - h->cur], 0, h->ncell);
         h->cur = 1 - h->cur;
      }
      if (st != LBM_OK) return st;
      h->t++;
   }
   return LBM_OK;
}

lbm_status lbm_get_macros(lbm_handle* h, double* rho, double* u)
{
   if (!h || !rho || !u) return LBM_ERR_INVALID_ARGUMENT;
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   // The reference reads AA through the streamed populations and AB straight
   // from the stored buffer (src/propagation/PropagationAB.cpp:222-281).
   const int mode = h->cfg.prop_pattern == LBM_PATTERN_AA ? logical_mode(h) : 0;
   lbm_status st = dense_for_read(h);
   if (st == LBM_OK) st = ensure_copy_stream(h);
   if (st != LBM_OK) return st;
   const int64_t n = h->ncell;
   const int64_t chunk = chunk_cells(h, 4);
   const size_t half = h->staging_elems / 2;
   const void* buf = readout_buffer(h);
   for (int64_t c0 = 0, k = 0; c0 < n; c0 += chunk, k++) {
      const int64_t cnt = std::min<int64_t>(chunk, n - c0);
      const int b = (int)(k & 1);
      double* part = h->staging + b * half;
      // the half is reused once its previous chunk has reached the host
      if (k >= 2) LBM_CUDA(h, cudaStreamWaitEvent(h->stream, h->chunk_free[b], 0));
      dispatch_q_st<Macros>(h->Q, h->storage, h, c0, cnt, buf, mode, part, part + cnt, cnt);
      LBM_CUDA(h, cudaGetLastError());
      LBM_CUDA(h, cudaEventRecord(h->chunk_ready[b], h->stream));
      LBM_CUDA(h, cudaStreamWaitEvent(h->copy_stream, h->chunk_ready[b], 0));
      LBM_CUDA(h, cudaMemcpyAsync(rho + c0, part, sizeof(double) * cnt, cudaMemcpyDeviceToHost, h->copy_stream));
      for (int d = 0; d < 3; d++)
         LBM_CUDA(h, cudaMemcpyAsync(u + (size_t)d * n + c0, part + (1 + d) * cnt, sizeof(double) * cnt,
                                     cudaMemcpyDeviceToHost, h->copy_stream));
      LBM_CUDA(h, cudaEventRecord(h->chunk_free[b], h->copy_stream));
   }
   cudaError_t e = cudaStreamSynchronize(h->copy_stream);
   if (e != cudaSuccess) return cuda_fail(h, e, "lbm_get_macros");
   return LBM_OK;
}

lbm_status lbm_reduce_conserved(lbm_handle* h, double out[4])
{
   if (!h || !out) return LBM_ERR_INVALID_ARGUMENT;
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   lbm_status st = dense_for_read(h);
   if (st != LBM_OK) return st;
   dispatch_q_st<Conserved>(h->Q, h->storage, h, readout_buffer(h), logical_mode(h), h->partials,
                            h->reduce_out);
   LBM_CUDA(h, cudaGetLastError());
   LBM_CUDA(h, cudaMemcpyAsync(out, h->reduce_out, sizeof(double) * 4, cudaMemcpyDeviceToHost, h->stream));
   LBM_CUDA(h, cudaStreamSynchronize(h->stream));
   for (int k = 0; k < 4; k++)
      if (!std::isfinite(out[k])) return fail(h, LBM_ERR_DIVERGED, "conserved sum %d is %g", k, out[k]);
   return LBM_OK;
}

static lbm_status check_range(lbm_handle* h, int64_t start, int64_t count)
{
   if (start < 0 || count < 0 || start + count > h->ncell)
      return fail(h, LBM_ERR_INVALID_ARGUMENT, "cell range [%lld, %lld) outside [0, %lld)", (long long)start,
                  (long long)(start + count), (long long)h->ncell);
   return LBM_OK;
}

lbm_status lbm_timestep_even_force(lbm_handle* h, void* dstrb, int64_t start, int64_t count)
{
   if (!h) return LBM_ERR_INVALID_ARGUMENT;
   if (!dstrb) return fail(h, LBM_ERR_INVALID_ARGUMENT, "null population buffer");
   if (h->cfg.prop_pattern != LBM_PATTERN_AA) return fail(h, LBM_ERR_STATE, "handle is not configured for AA");
   lbm_status st = check_range(h, start, count);
   if (st != LBM_OK) return st;
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   return launch(h, K_AA_EVEN, dstrb, dstrb, start, count);
}

lbm_status lbm_timestep_odd_force(lbm_handle* h, void* dstrb, int64_t start, int64_t count)
{
   if (!h) return LBM_ERR_INVALID_ARGUMENT;
   if (!dstrb) return fail(h, LBM_ERR_INVALID_ARGUMENT, "null population buffer");
   if (h->cfg.prop_pattern != LBM_PATTERN_AA) return fail(h, LBM_ERR_STATE, "handle is not configured for AA");
   lbm_status st = check_range(h, start, count);
   if (st != LBM_OK) return st;
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   return launch(h, K_AA_ODD, dstrb, dstrb, start, count);
}

lbm_status lbm_timestep_force(lbm_handle* h, const void* src, void* tgt, int64_t start, int64_t count)
{
   if (!h) return LBM_ERR_INVALID_ARGUMENT;
   if (h->cfg.prop_pattern != LBM_PATTERN_AB) return fail(h, LBM_ERR_STATE, "handle is not configured for AB");
   if (!src || !tgt) return fail(h, LBM_ERR_INVALID_ARGUMENT, "null population buffer");
   if (src == tgt) return fail(h, LBM_ERR_INVALID_ARGUMENT, "AB needs two distinct buffers");
   lbm_status st = check_range(h, start, count);
   if (st != LBM_OK) return st;
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   return launch(h, h->cfg.pull ? K_AB_PULL : K_AB_PUSH, src, tgt, start, count);
}

lbm_status lbm_copy_state(lbm_handle* h, void* dev, int to_handle)
{
   if (!h || !dev) return LBM_ERR_INVALID_ARGUMENT;
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   void* buf = const_cast<void*>(readout_buffer(h));
   if (to_handle) {
      LBM_CUDA(h, cudaMemcpyAsync(buf, dev, h->buffer_bytes, cudaMemcpyDeviceToDevice, h->stream));
      dense_written(h);
   } else {
      lbm_status st = dense_for_read(h);
      if (st != LBM_OK) return st;
      LBM_CUDA(h, cudaMemcpyAsync(dev, buf, h->buffer_bytes, cudaMemcpyDeviceToDevice, h->stream));
   }
   return LBM_OK;
}

namespace {
__global__ void d2f_kernel(const double* src, float* dst, int64_t n)
{
   const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
   if (i < n) dst[i] = (float)src[i];
}
}  // namespace

static lbm_status set_field_device(lbm_handle* h, const double* dev, int ncomp, double** d64, float** d32)
{
   const size_t n = (size_t)h->plane * ncomp;
   if (!dev) {
      dev_free(h, *d64, sizeof(double) * n);
      dev_free(h, *d32, sizeof(float) * n);
      *d64 = nullptr;
      *d32 = nullptr;
      return LBM_OK;
   }
   if (h->storage == ST_F64) {
      if (!*d64) {
         lbm_status st = dev_alloc(h, (void**)d64, sizeof(double) * n);
         if (st != LBM_OK) return st;
      }
      LBM_CUDA(h, cudaMemcpyAsync(*d64, dev, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
   } else {
      if (!*d32) {
         lbm_status st = dev_alloc(h, (void**)d32, sizeof(float) * n);
         if (st != LBM_OK) return st;
      }
      d2f_kernel<<<blocks_for((int64_t)n, 256), 256, 0, h->stream>>>(dev, *d32, (int64_t)n);
      LBM_CUDA(h, cudaGetLastError());
      // the adjoint reads FP64 fields whatever the storage
      if (!*d64) {
         lbm_status st = dev_alloc(h, (void**)d64, sizeof(double) * n);
         if (st != LBM_OK) return st;
      }
      LBM_CUDA(h, cudaMemcpyAsync(*d64, dev, sizeof(double) * n, cudaMemcpyDeviceToDevice, h->stream));
   }
   return LBM_OK;
}

lbm_status lbm_set_fields_device(lbm_handle* h, const double* force_field, const double* porosity)
{
   if (!h) return LBM_ERR_INVALID_ARGUMENT;
   if (h->compact && (force_field || porosity))
      return fail(h, LBM_ERR_UNSUPPORTED, "compact storage has no per-cell fields");
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   lbm_status st = set_field_device(h, force_field, 3, &h->force_field, &h->force_field_f);
   if (st == LBM_OK) st = set_field_device(h, porosity, 1, &h->porosity, &h->porosity_f);
   return st;
}

static AdjParams adj_params(const lbm_handle* h, const void* state)
{
   AdjParams a;
   std::memset(&a, 0, sizeof(a));
   a.g = dims_of(h);
   a.omega = h->cfg.omega;
   for (int d = 0; d < 3; d++) a.F[d] = h->cfg.force[d];
   a.links = h->links;
   a.force_field = h->force_field;
   a.porosity = h->porosity;
   a.state = state ? state : readout_buffer(h);
   return a;
}

lbm_status lbm_loss(lbm_handle* h, const void* state, int loss_kind, const double* weight, double time_weight,
                    double* out_host)
{
   if (!h || !weight || !out_host || (loss_kind != LBM_LOSS_VELOCITY && loss_kind != LBM_LOSS_ENERGY))
      return LBM_ERR_INVALID_ARGUMENT;
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   if (!state) {
      lbm_status st = dense_for_read(h);
      if (st != LBM_OK) return st;
   }
   AdjParams a = adj_params(h, state);
   a.loss_kind = loss_kind;
   a.loss_weight = weight;
   a.time_weight = time_weight;
   LBM_CUDA(h, launch_loss(h->Q, h->storage, a, h->partials, kReduceBlocks, h->reduce_out, h->stream));
   LBM_CUDA(h, cudaMemcpyAsync(out_host, h->reduce_out, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
   LBM_CUDA(h, cudaStreamSynchronize(h->stream));
   return LBM_OK;
}

lbm_status lbm_adjoint_step(lbm_handle* h, const void* state, const double* lam_next, double* lam, int collide,
                            int loss_kind, const double* weight, double time_weight, double* grad_force,
                            double* grad_porosity)
{
   if (!h || !state || !lam || (collide && !lam_next)) return LBM_ERR_INVALID_ARGUMENT;
   if (h->cfg.prop_pattern != LBM_PATTERN_AB || h->cfg.pull)
      return fail(h, LBM_ERR_STATE, "the adjoint differentiates AB-push rollouts");
   if (loss_kind != LBM_LOSS_NONE && !weight) return LBM_ERR_INVALID_ARGUMENT;
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   AdjParams a = adj_params(h, state);
   a.lam_next = lam_next;
   a.lam = lam;
   a.collide = collide;
   a.loss_kind = loss_kind;
   a.loss_weight = weight;
   a.time_weight = time_weight;
   a.grad_force = grad_force;
   a.grad_porosity = grad_porosity;
   LBM_CUDA(h, launch_adjoint(h->Q, h->storage, a, h->stream));
   return LBM_OK;
}

lbm_status lbm_adjoint_step_f32(lbm_handle* h, const void* state, const float* lam_next, float* lam, int collide,
                                int loss_kind, const double* weight, double time_weight, double* grad_force,
                                double* grad_porosity)
{
   if (!h || !state || !lam || (collide && !lam_next)) return LBM_ERR_INVALID_ARGUMENT;
   if (h->cfg.prop_pattern != LBM_PATTERN_AB || h->cfg.pull)
      return fail(h, LBM_ERR_STATE, "the adjoint differentiates AB-push rollouts");
   if (loss_kind != LBM_LOSS_NONE && !weight) return LBM_ERR_INVALID_ARGUMENT;
   LBM_CUDA(h, cudaSetDevice(h->cfg.device));
   AdjParams a = adj_params(h, state);
   a.lam_next_f = lam_next;
   a.lam_f = lam;
   a.collide = collide;
   a.loss_kind = loss_kind;
   a.loss_weight = weight;
   a.time_weight = time_weight;
   a.grad_force = grad_force;
   a.grad_porosity = grad_porosity;
   LBM_CUDA(h, launch_adjoint_f32(h->Q, h->storage, a, h->stream));
   return LBM_OK;
}

lbm_status lbm_population_buffer(lbm_handle* h, void** dev_ptr)
{
   if (!h || !dev_ptr) return LBM_ERR_INVALID_ARGUMENT;
   if (h->compact)
      return fail(h, LBM_ERR_UNSUPPORTED, "compact storage keeps its state in the compact buffer, not a dense one");
   *dev_ptr = const_cast<void*>(readout_buffer(h));
   return LBM_OK;
}

}  // extern "C"
