// Propagation-level shim: one GB300 library handle in place of the reference's
// PropagationAA / PropagationAB (src/propagation/Propagation.hh:9-55).  The
// handle owns the device buffers; the geometry comes from the reference's own
// Geometry (its grid marks walls with negative values), so Main.cpp only has to
// construct this class instead of PropagationAA/AB, e.g. behind an input key.
//
// Selected settings follow the reference's keys: propPattern (AA or AB), pull,
// unroll (KernelAA_SOA_Unroll's rest forcing weight), _OMEGA_, _GRAVITY_.  One
// rank: the domain wraps in x only, as GeometryAAAB::setupAdjacency does on one
// rank (src/geometries/GeometryAAAB.cpp:56-66).
#ifndef PROPAGATION_GB300_HH
#define PROPAGATION_GB300_HH

#include <mpi.h>

#include <cstdint>
#include <vector>

#include "Propagation.hh"
#include "gb300_check.hh"
#include "lbm_gb300.h"

class PropagationGB300 : public Propagation
{
public:
   PropagationGB300(Lattice& lattice, Geometry& geometry, Communication& comm, Parameters& parameters)
      : Propagation(lattice, geometry, comm, parameters)
   {
   }
   ~PropagationGB300() override { lbm_destroy(h_); }

   void setup() override
   {
      L_[0] = geometry_.getTotalLengthByDim(0);
      L_[1] = geometry_.getTotalLengthByDim(1);
      L_[2] = geometry_.getTotalLengthByDim(2);
      lbm_config cfg;
      gb300_check(lbm_config_default(&cfg), "lbm_config_default", nullptr);
      cfg.lattice = _LATTICESIZE_;
      cfg.prop_pattern = parameters_.getPropPattern() == 1 ? LBM_PATTERN_AA : LBM_PATTERN_AB;
      cfg.pull = parameters_.getPullSetting();
      cfg.unroll = parameters_.getUnrollSetting();
      cfg.nx = L_[0];
      cfg.ny = L_[1];
      cfg.nz = L_[2];
      cfg.periodic[0] = 1;
      cfg.periodic[1] = 0;
      cfg.periodic[2] = 0;
      cfg.omega = _OMEGA_;
      cfg.force[0] = _GRAVITY_;
      gb300_check(lbm_create(&cfg, &h_), "lbm_create", nullptr);
      // the reference's grid is k fastest, the library's x fastest
      std::vector<uint8_t> solid(ncell());
      for (int i = 0; i < L_[0]; i++)
         for (int j = 0; j < L_[1]; j++)
            for (int k = 0; k < L_[2]; k++)
               solid[dense(i, j, k)] = geometry_.getGridElement(geometry_.getGridIdx(i, j, k)) < 0;
      gb300_check(lbm_set_solid(h_, solid.data()), "lbm_set_solid", lbm_last_error(h_));
   }

   void initialize() override
   {
      gb300_check(lbm_init_equilibrium(h_, nullptr, nullptr), "lbm_init_equilibrium", lbm_last_error(h_));
   }

   void run() override
   {
      initialize();
      MPI_Barrier(MPI_COMM_WORLD);
      const double t0 = MPI_Wtime();
      gb300_check(lbm_step(h_, parameters_.getTimesteps()), "lbm_step", lbm_last_error(h_));
      gb300_check(lbm_synchronize(h_), "lbm_synchronize", lbm_last_error(h_));
      const double t1 = MPI_Wtime();
      if (myRank_ == 0) printMFLUPS(t1 - t0);
      rho_.resize(ncell());
      u_.resize(3 * ncell());
      gb300_check(lbm_get_macros(h_, rho_.data(), u_.data()), "lbm_get_macros", lbm_last_error(h_));
      checkResult(parameters_.getTimesteps());
   }

   // readouts keyed by the reference's fluid index, after run()
   Pdf getRho(int fluidIdx, int) override { return rho_[dense_of_fluid(fluidIdx)]; }
   vector<Pdf> getVelocity(int fluidIdx, int) override
   {
      const size_t c = dense_of_fluid(fluidIdx);
      return {u_[c], u_[ncell() + c], u_[2 * ncell() + c]};
   }

   lbm_handle* handle() { return h_; }

private:
   size_t ncell() const { return (size_t)L_[0] * L_[1] * L_[2]; }
   size_t dense(int i, int j, int k) const { return i + (size_t)L_[0] * (j + (size_t)L_[1] * k); }
   size_t dense_of_fluid(int f) const
   {
      const vector<int>& p = geometry_.fluidPts_[f];
      return dense(p[0], p[1], p[2]);
   }

   lbm_handle* h_ = nullptr;
   int L_[3] = {0, 0, 0};
   vector<double> rho_, u_;
};

#endif
