// Kernel-level shims on the reference's own compact buffers: dstrb[nFluid*s + i]
// with the fluid points in the reference's sorted order, streamed through the
// adjacency list GeometryAAAB::setupAdjacency already built
// (src/geometries/GeometryAAAB.cpp:18-124).  The reference keeps its Geometry,
// Propagation, fluid ordering and border/bulk ranges; only the population
// buffers must live in device memory (a CUDA allocation where the reference
// calls new Pdf[]).  The classes implement src/kernels/KernelAA.hh:7-58 and
// src/kernels/KernelAB.hh:8-50; the steps run asynchronously on the handle's
// stream (lbm_sparse_set_stream), so the driver synchronises where the
// reference's SYCL path waits on its queue.
#ifndef KERNEL_GB300_COMPACT_HH
#define KERNEL_GB300_COMPACT_HH

#include "KernelAA.hh"
#include "KernelAB.hh"
#include "gb300_check.hh"
#include "lbm_gb300.h"

inline lbm_sparse_handle* gb300_sparse_handle(Geometry& g, Parameters& p)
{
   lbm_config cfg;
   gb300_check(lbm_config_default(&cfg), "lbm_config_default", nullptr);
   cfg.lattice = _LATTICESIZE_;
   cfg.prop_pattern = p.getPropPattern() == 1 ? LBM_PATTERN_AA : LBM_PATTERN_AB;
   cfg.pull = p.getPullSetting();
   cfg.unroll = p.getUnrollSetting();   // KernelAA_SOA_Unroll's rest forcing weight
   cfg.omega = _OMEGA_;
   cfg.force[0] = _GRAVITY_;
   lbm_sparse_handle* h = nullptr;
   gb300_check(lbm_sparse_create(&cfg, g.getNumFluidPts(), g.adjacency_, &h), "lbm_sparse_create", nullptr);
   return h;
}

class KernelAA_GB300Compact : public KernelAA
{
public:
   KernelAA_GB300Compact(Lattice& lattice, Geometry& geometry, Parameters& parameters)
      : KernelAA(lattice, geometry), h_(gb300_sparse_handle(geometry, parameters))
   {
   }
   ~KernelAA_GB300Compact() override { lbm_sparse_destroy(h_); }
   void setup() override {}
   void timestepEvenForce(Pdf* dstrb, int startIdx, int countIdx) override
   {
      gb300_check(lbm_sparse_timestep_even_force(h_, dstrb, startIdx, countIdx), "timestepEvenForce",
                  lbm_sparse_last_error(h_));
   }
   void timestepOddForce(Pdf* dstrb, int startIdx, int countIdx) override
   {
      gb300_check(lbm_sparse_timestep_odd_force(h_, dstrb, startIdx, countIdx), "timestepOddForce",
                  lbm_sparse_last_error(h_));
   }
   lbm_sparse_handle* handle() { return h_; }

private:
   lbm_sparse_handle* h_;
};

// Push or pull per the input key "pull"; the adjacency must be the one
// GeometryAAAB built for that setting.
class KernelAB_GB300Compact : public KernelAB
{
public:
   KernelAB_GB300Compact(Lattice& lattice, Geometry& geometry, Parameters& parameters)
      : KernelAB(lattice, geometry), h_(gb300_sparse_handle(geometry, parameters))
   {
   }
   ~KernelAB_GB300Compact() override { lbm_sparse_destroy(h_); }
   void setup() override {}
   void timestepForce(Pdf* dstrb_src, Pdf* dstrb_tgt, int startIdx, int countIdx) override
   {
      gb300_check(lbm_sparse_timestep_force(h_, dstrb_src, dstrb_tgt, startIdx, countIdx), "timestepForce",
                  lbm_sparse_last_error(h_));
   }
   lbm_sparse_handle* handle() { return h_; }

private:
   lbm_sparse_handle* h_;
};

#endif
