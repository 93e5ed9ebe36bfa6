// Compact fluid-only layout for the shifted FP32 / BF16 / FP16 storage (AA
// propagation): populations exist only for fluid cells, numbered in the
// dense grid's order (x fastest, then y, then z) with the solid cells left
// out, direction s of fluid cell i at s * cplane + i.
//
// Streaming needs no per-direction adjacency list.  A row r = y + ny z holds
// its fluid cells at consecutive indices from rows[r].start, and pre[c] counts
// the fluid cells of c's row that lie before c; so the fluid cell at (x', r')
// is rows[r'].start + pre[x' + nx r'].  A lane of row r at x needs, for each
// of the 9 rows r' = r + (dy, dz), one value base = rows[r'].start +
// pre[x + nx r'] (its own row: its own index i); the neighbours at x - 1,
// x and x + 1 of that row are base - 1, base and base + [x fluid in r'], with
// the periodic wrap of x folded in through the row's fluid count.  Whether a
// neighbour is fluid comes from the cell's link word, as in the dense layout
// (bit s set: the neighbour at x + c_s is solid or outside a non-periodic
// face).  This costs 2 bytes per dense cell (pre) and 6 per fluid cell (x and
// the link word), against the 4 Q bytes per fluid cell of an adjacency list.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "lbm_physics.cuh"

namespace lbm {

struct RowInfo {
   uint32_t start;   // compact index of the row's first fluid cell
   uint32_t count;   // fluid cells in the row
};

struct CompactGeom {
   const uint32_t* tile_first;   // [nrow_tiles] first compact index of a row tile (up to 32 cells of one row)
   const uint32_t* tile_row;     // [nrow_tiles] its row y + ny z
   const RowInfo* rows;          // [ny nz]
   const uint16_t* pre;          // [ncell] fluid cells before x in the cell's row
   const uint16_t* xs;           // [nf] x of each fluid cell
   const uint32_t* lk;           // [nf] link word of each fluid cell
   uint32_t nrow_tiles;
   uint32_t nf;                  // fluid cells
   uint32_t cplane;              // elements between direction planes (even, at least nf)
   int nx, ny, nz;
   uint64_t m_ny;                // ceil(2^64 / ny), 0 for ny = 1: row -> (y, z) by multiply-high
   uint32_t soff[27];            // s * cplane: slot offsets in the parameter bank
};

// One AA step (kind K_AA_EVEN or K_AA_ODD) on a compact buffer.
cudaError_t launch_compact_step(int Q, int storage, int kind, const KParams& p, const CompactGeom& g, void* buf,
                                cudaStream_t stream);
// Dense <-> compact copies of a whole population buffer (raw layout, the same
// slot contents): dense slot s of cell dcell[i] <-> compact slot s of fluid
// cell i.
cudaError_t launch_compact_expand(int Q, int storage, const uint32_t* dcell, uint32_t nf, uint32_t cplane,
                                  const void* cbuf, void* dense, int64_t plane, cudaStream_t stream);
cudaError_t launch_compact_compress(int Q, int storage, const uint32_t* dcell, uint32_t nf, uint32_t cplane,
                                    const void* dense, int64_t plane, void* cbuf, cudaStream_t stream);
// lk[i] = links[dcell[i]]
cudaError_t launch_compact_links(const uint32_t* dcell, const uint32_t* links, uint32_t* lk, uint32_t nf,
                                 cudaStream_t stream);

}  // namespace lbm
