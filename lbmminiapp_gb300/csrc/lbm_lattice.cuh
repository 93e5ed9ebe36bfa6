// Compile-time D3Q19 / D3Q27 velocity sets for device code.
//
// Direction order, opposite table and weights are the reference's
// (src/lattices/LatticeD3Q19.cpp:5-88, src/lattices/LatticeD3Q27.cpp:5-120):
// the slot order is part of the raw population layout shared with callers,
// so it must be the same.  Everything here folds to constants once the
// direction loops are unrolled.
#pragma once

#include <cstdint>

namespace lbm {

__host__ __device__ constexpr int lat_c(int Q, int s, int d)
{
   constexpr int c19[19][3] = {
      {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
      {1, 1, 0}, {1, -1, 0}, {1, 0, 1}, {1, 0, -1}, {-1, 1, 0}, {-1, -1, 0},
      {-1, 0, 1}, {-1, 0, -1}, {0, 1, 1}, {0, 1, -1}, {0, -1, 1}, {0, -1, -1},
      {0, 0, 0}};
   constexpr int c27[27][3] = {
      {1, 0, 0}, {-1, 0, 0}, {0, 1, 0}, {0, -1, 0}, {0, 0, 1}, {0, 0, -1},
      {1, 1, 0}, {1, -1, 0}, {1, 0, 1}, {1, 0, -1}, {-1, 1, 0}, {-1, -1, 0},
      {-1, 0, 1}, {-1, 0, -1}, {0, 1, 1}, {0, 1, -1}, {0, -1, 1}, {0, -1, -1},
      {1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {1, -1, -1}, {-1, 1, 1}, {-1, 1, -1},
      {-1, -1, 1}, {-1, -1, -1}, {0, 0, 0}};
   return Q == 19 ? c19[s][d] : c27[s][d];
}

__host__ __device__ constexpr int lat_opp(int Q, int s)
{
   constexpr int o19[19] = {1, 0, 3, 2, 5, 4, 11, 10, 13, 12, 7, 6, 9, 8, 17, 16, 15, 14, 18};
   constexpr int o27[27] = {1, 0, 3, 2, 5, 4, 11, 10, 13, 12, 7, 6, 9, 8, 17, 16,
                            15, 14, 25, 24, 23, 22, 21, 20, 19, 18, 26};
   return Q == 19 ? o19[s] : o27[s];
}

__host__ __device__ constexpr int lat_norm2(int Q, int s)
{
   return lat_c(Q, s, 0) * lat_c(Q, s, 0) + lat_c(Q, s, 1) * lat_c(Q, s, 1) +
          lat_c(Q, s, 2) * lat_c(Q, s, 2);
}

// Weights as correctly rounded doubles, the values the reference's
// Lattice::stencil_[s].c divisions produce (1.0/18.0 etc.).
__host__ __device__ constexpr double lat_w(int Q, int s)
{
   return Q == 19 ? (lat_norm2(Q, s) == 0 ? 1.0 / 3.0
                                          : (lat_norm2(Q, s) == 1 ? 1.0 / 18.0 : 1.0 / 36.0))
                  : (lat_norm2(Q, s) == 0
                        ? 8.0 / 27.0
                        : (lat_norm2(Q, s) == 1 ? 2.0 / 27.0
                                                : (lat_norm2(Q, s) == 2 ? 1.0 / 54.0 : 1.0 / 216.0)));
}

__host__ __device__ constexpr int lat_rest(int Q) { return Q - 1; }

}  // namespace lbm
