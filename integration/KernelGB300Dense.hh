// Kernel-level shims on buffers in the library's dense layout, for a driver
// that keeps its own Propagation: lbm_info.plane_stride elements per direction,
// lbm_info.buffer_bytes per buffer, cell index x + nx*(y + ny*z), and
// startIdx/countIdx a range of dense cell indices (solid cells in it are
// skipped).  The handle (lbm_create + lbm_set_solid) carries the lattice,
// pattern, relaxation rate, force and geometry.  Implements
// src/kernels/KernelAA.hh:7-58 and src/kernels/KernelAB.hh:8-50.
#ifndef KERNEL_GB300_DENSE_HH
#define KERNEL_GB300_DENSE_HH

#include "KernelAA.hh"
#include "KernelAB.hh"
#include "gb300_check.hh"
#include "lbm_gb300.h"

class KernelAA_GB300 : public KernelAA
{
public:
   KernelAA_GB300(Lattice& lattice, Geometry& geometry, lbm_handle* h) : KernelAA(lattice, geometry), h_(h) {}
   void setup() override {}
   void timestepEvenForce(Pdf* dstrb, int startIdx, int countIdx) override
   {
      gb300_check(lbm_timestep_even_force(h_, dstrb, startIdx, countIdx), "timestepEvenForce", lbm_last_error(h_));
   }
   void timestepOddForce(Pdf* dstrb, int startIdx, int countIdx) override
   {
      gb300_check(lbm_timestep_odd_force(h_, dstrb, startIdx, countIdx), "timestepOddForce", lbm_last_error(h_));
   }

private:
   lbm_handle* h_;
};

class KernelAB_GB300 : public KernelAB
{
public:
   KernelAB_GB300(Lattice& lattice, Geometry& geometry, lbm_handle* h) : KernelAB(lattice, geometry), h_(h) {}
   void setup() override {}
   void timestepForce(Pdf* dstrb_src, Pdf* dstrb_tgt, int startIdx, int countIdx) override
   {
      gb300_check(lbm_timestep_force(h_, dstrb_src, dstrb_tgt, startIdx, countIdx), "timestepForce",
                  lbm_last_error(h_));
   }

private:
   lbm_handle* h_;
};

#endif
