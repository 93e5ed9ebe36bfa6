// Host build of the compact layout's set-up (lbmminiapp_gb300/csrc/
// lbm_compact_tiles.hh) for tests/test_compact_host.py: the fluid numbering
// and the odd step's row tiles for a mask, without a GPU.
#include <cstring>

#include "lbm_compact_tiles.hh"

// Fills dcell [nfluid], tiles [ntiles * 20 words] and u [ntiles * 64 words]
// when they hold cap_cells / cap_tiles entries; returns 0, or -1 with the
// sizes set when they do not.
extern "C" int compact_tiles_host(int nx, int ny, int nz, const uint8_t* solid, uint32_t* dcell, uint32_t* tiles,
                                  uint32_t* u, long long cap_cells, long long cap_tiles, long long* nfluid,
                                  long long* ntiles)
{
   std::vector<uint32_t> d, uc;
   std::vector<lbm::OddTile> t;
   lbm::build_row_tiles(nx, ny, nz, solid, d, t, uc);
   *nfluid = (long long)d.size();
   *ntiles = (long long)t.size();
   if ((long long)d.size() > cap_cells || (long long)t.size() > cap_tiles) return -1;
   std::memcpy(dcell, d.data(), 4 * d.size());
   std::memcpy(tiles, t.data(), sizeof(lbm::OddTile) * t.size());
   std::memcpy(u, uc.data(), 4 * uc.size());
   return 0;
}
