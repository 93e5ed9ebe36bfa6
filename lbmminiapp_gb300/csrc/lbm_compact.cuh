// Compact fluid-only layout for the shifted FP32 / BF16 / FP16 storage (AA
// propagation): populations exist only for fluid cells, numbered in the
// dense grid's order (x fastest, then y, then z) with the solid cells left
// out, direction s of fluid cell i at s * cplane + i.
//
// Streaming needs no per-direction adjacency list.  The odd step works on
// row tiles: up to 32 consecutive fluid cells of one row r = y + ny z whose x
// lie at most 255 past the tile's first x (xa).  Per tile, for each of the 9 rows
// r' = r + (dy, dz) (periodic wrap of y and z), b[k] is the compact index of
// the first fluid cell of r' at or after xa and n[k] the fluid count of r';
// per cell, u[k] counts the fluid cells of r' in [xa, x).  The fluid cell at
// (x, r') is then b[k] + u[k], its neighbours at x - 1 and x + 1 are one below
// and one past it (past it only when (x, r') is fluid), and at the row ends
// the periodic wrap of x adds or takes off n[k].  Whether a neighbour is fluid
// comes from the cell's link word, as in the dense layout (bit s set: the
// neighbour at x + c_s is solid or outside a non-periodic face).  This costs
// 80 bytes per tile and 12 per cell (the 8 counts u[k] of the other rows and
// the link word), against the 4 Q bytes per fluid cell of an adjacency list,
// and every one of it is read with the cell's own index: no load of the odd
// step depends on another.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "lbm_compact_tiles.hh"
#include "lbm_physics.cuh"

namespace lbm {

// Link-word bits of a compact cell beyond the direction bits (Q <= 27) and
// kSolidBit (a tile lane without a cell): the cell sits at x = 0 / x = nx - 1.
constexpr uint32_t kRowStartBit = 1u << 29;
constexpr uint32_t kRowEndBit = 1u << 30;

struct CompactGeom {
   const OddTile* tiles;         // [nrow_tiles]
   const uint2* u;               // [nrow_tiles * 32] bytes u[k] of rows k = 0..3, 5..8 per tile lane
   const uint32_t* lk;           // [nrow_tiles * 32] link word of each tile lane (kSolidBit: no cell)
   uint32_t nrow_tiles;
   uint32_t nf;                  // fluid cells
   uint32_t cplane;              // elements between direction planes (even, at least nf)
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
// Link words of the tile lanes: links[dcell[i]] (0 without links) with the
// row-end bits for the cell i of each lane, kSolidBit for a lane past its
// tile's cells.
cudaError_t launch_compact_links(const OddTile* tiles, uint32_t ntiles, const uint32_t* dcell,
                                 const uint32_t* links, int nx, uint32_t* lk, cudaStream_t stream);

}  // namespace lbm
