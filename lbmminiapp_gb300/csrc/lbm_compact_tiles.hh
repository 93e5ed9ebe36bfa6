// Host-side set-up of the compact fluid-only layout (lbm_compact.cuh): the
// compact numbering of the fluid cells and the row tiles of the AA odd step.
// Plain C++ (no CUDA types), so the same code is built into the library and
// into the CPU tests (tests/native/compact_tiles_check.cpp).
#pragma once

#include <cstdint>
#include <vector>

namespace lbm {

// Row tile of the odd step, 80 bytes (five 16-byte copies).
struct OddTile {
   uint32_t b[9];       // compact index of the first fluid cell at or after xa in row k = 3 (dy + 1) + (dz + 1)
   uint32_t n[9];       // fluid cells in row k
   uint32_t ncell;      // fluid cells in the tile (1..32)
   uint32_t pad;
};
static_assert(sizeof(OddTile) == 80, "OddTile is five 16-byte words");

// The fluid cells of an nx x ny x nz grid (solid: dense mask, x fastest, null
// for all fluid), numbered in the dense order with the solids left out:
// dcell[i] is the dense cell of fluid cell i.  The odd step's row tiles: up to
// 32 consecutive fluid cells of one row r = y + ny z whose x lie at most 255
// past the first one's (xa).  Per tile, the compact index b[k] of the first
// fluid cell at or after xa in each neighbour row r + (dy, dz) (y and z wrap)
// and that row's fluid count n[k]; per tile lane, two words of byte-sized
// counts u[k] of fluid cells of row k in [xa, x) for k = 0..3, 5..8 (bytes 0-3
// of the first word, then of the second), zero past the tile's cells.
inline void build_row_tiles(int nx, int ny, int nz, const uint8_t* solid, std::vector<uint32_t>& dcell,
                            std::vector<OddTile>& tiles, std::vector<uint32_t>& ucounts)
{
   const int64_t nrows = (int64_t)ny * nz;
   // per row: first compact index and fluid count; per cell: fluid cells
   // before it in its row
   std::vector<uint32_t> rstart((size_t)nrows), rcount((size_t)nrows);
   std::vector<uint16_t> pre((size_t)(nrows * nx));
   dcell.clear();
   for (int64_t r = 0; r < nrows; r++) {
      rstart[(size_t)r] = (uint32_t)dcell.size();
      uint32_t cnt = 0;
      for (int x = 0; x < nx; x++) {
         const int64_t c = r * nx + x;
         pre[(size_t)c] = (uint16_t)cnt;
         if (!solid || !solid[c]) {
            dcell.push_back((uint32_t)c);
            cnt++;
         }
      }
      rcount[(size_t)r] = cnt;
   }
   tiles.clear();
   ucounts.clear();
   tiles.reserve(dcell.size() / 32 + (size_t)nrows);
   ucounts.reserve(2 * (dcell.size() + (size_t)nrows * 32));
   for (int64_t r = 0; r < nrows; r++) {
      const int y = (int)(r % ny), z = (int)(r / ny);
      int64_t nbr[9];
      for (int k = 0; k < 9; k++) {
         const int yy = (y + k / 3 - 1 + ny) % ny, zz = (z + k % 3 - 1 + nz) % nz;
         nbr[k] = (int64_t)yy + (int64_t)ny * zz;
      }
      const uint32_t start = rstart[(size_t)r], cnt = rcount[(size_t)r];
      uint32_t q = 0;
      while (q < cnt) {
         const int xa = (int)(dcell[start + q] - (uint32_t)(r * nx));
         OddTile t{};
         for (int k = 0; k < 9; k++) {
            const int64_t rk = nbr[k];
            t.b[k] = rstart[(size_t)rk] + pre[(size_t)(rk * nx + xa)];
            t.n[k] = rcount[(size_t)rk];
         }
         uint32_t m = 0;
         while (m < 32 && q + m < cnt) {
            const int x = (int)(dcell[start + q + m] - (uint32_t)(r * nx));
            if (x - xa > 255) break;
            uint32_t w[2] = {0u, 0u};
            int byte = 0;
            for (int k = 0; k < 9; k++) {
               if (k == 4) continue;
               const int64_t rk = nbr[k];
               const uint32_t uk = (uint32_t)pre[(size_t)(rk * nx + x)] - pre[(size_t)(rk * nx + xa)];
               w[byte / 4] |= uk << (8 * (byte % 4));
               byte++;
            }
            ucounts.push_back(w[0]);
            ucounts.push_back(w[1]);
            m++;
         }
         t.ncell = m;
         for (uint32_t l = m; l < 32; l++) {
            ucounts.push_back(0u);
            ucounts.push_back(0u);
         }
         tiles.push_back(t);
         q += m;
      }
   }
}

}  // namespace lbm
