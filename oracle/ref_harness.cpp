/*
 * Test-only harness around the UNMODIFIED lbmminiapp CPU kernels.
 *
 * Built by oracle/build_ref.sh from the reference's own sources (lattices,
 * Geometry, GeometryAAAB, kernels, Propagation*, Communication, Parameters)
 * into oracle/_ref/libref_q{19,27}.so.  Nothing in the product library links
 * or loads it; tests use it to pin the C restatement (oracle/lbm_oracle.c)
 * and the golden fixtures against the reference itself.
 *
 * Two entry points:
 *
 *  ref_box_run   -- drives the reference kernel classes on a dense box with a
 *                   solid mask and per-axis periodicity.  The reference's own
 *                   GeometryAAAB can only build its cylinder and wraps only x
 *                   on one rank (src/geometries/GeometryAAAB.cpp:56-66), so a
 *                   harness Geometry subclass fills the same protected members
 *                   and builds the adjacency with the semantics of
 *                   GeometryAAAB::setupAdjacency (:44-84): the neighbour is
 *                   x+c_s for AB push, x-c_s for AA and AB pull; a wall or
 *                   out-of-box neighbour maps to the own cell's opp(s) slot;
 *                   each periodic axis wraps.
 *
 *  ref_app_*     -- runs the reference's complete single-rank flow
 *                   (src/Main.cpp:45-126) on one of its own input files:
 *                   Parameters, GeometryAAAB cylinder, Communication,
 *                   PropagationAA/AB setup + run (which print the MFLUPS and
 *                   validation lines), then reads rho/u back through the
 *                   reference's getRho/getVelocity.
 */
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

#include "Communication.hh"
#include "Geometry.hh"
#include "GeometryAAAB.hh"
#include "KernelAA_SOA_Base.hh"
#include "KernelAA_SOA_Unroll.hh"
#include "KernelAB_SOA_Base.hh"
#include "KernelAB_SOA_Pull.hh"
#include "KernelAB_SOA_Unroll.hh"
#include "KernelAB_SOA_Unroll_Pull.hh"
#include "Lattice.hh"
#include "LatticeD3Q19.hh"
#include "LatticeD3Q27.hh"
#include "Parameters.hh"
#include "PropagationAA.hh"
#include "PropagationAB.hh"

double lbm_ref_omega = 1.0;
double lbm_ref_gravity = 0.000001;

namespace {

Lattice* make_lattice()
{
   if (_LATTICESIZE_ == 27) return new LatticeD3Q27;
   return new LatticeD3Q19;
}

/* Dense box geometry with the reference's member layout (grid index k fastest,
 * src/geometries/Geometry.cpp:170-185) and a lexicographic fluid order. */
class HarnessGeometry : public Geometry
{
public:
   HarnessGeometry(Lattice& lattice, Parameters& parameters, int nx, int ny, int nz,
                   const unsigned char* solid, const int* periodic, bool pushNeighbour)
      : Geometry(lattice, parameters), push_(pushNeighbour)
   {
      dims_[0] = nx; dims_[1] = ny; dims_[2] = nz;
      for (int d = 0; d < 3; d++) periodic_[d] = periodic ? periodic[d] : 1;
      totalLength_ = {nx, ny, nz};
      myMin_ = {0, 0, 0};
      myMax_ = {nx - 1, ny - 1, nz - 1};
      myDims_ = {nx, ny, nz};
      boxes_ = {1, 1, 1};
      grid_.assign((size_t)nx * ny * nz, LAT_PT_WALL);
      for (int i = 0; i < nx; i++)
         for (int j = 0; j < ny; j++)
            for (int k = 0; k < nz; k++) {
               size_t dense = (size_t)i + (size_t)nx * ((size_t)j + (size_t)ny * k);
               if (solid && solid[dense]) continue;
               fluidPts_.push_back({i, j, k});
            }
      nFluid_ = (int)fluidPts_.size();
      nFluidGlobal_ = nFluid_;
      startInlet_ = countInlet_ = 0;
      startOutlet_ = countOutlet_ = 0;
      startBorder_ = countBorder_ = 0;
      startBulk_ = 0;
      countBulk_ = nFluid_;
      for (int f = 0; f < nFluid_; f++) {
         grid_[getGridIdx(fluidPts_[f][0], fluidPts_[f][1], fluidPts_[f][2])] = f;
      }
   }

   void setup() override {}

   void setupAdjacency() override
   {
      const int Q = _LATTICESIZE_;
      adjacency_ = new int[(size_t)nFluid_ * Q];
      for (int f = 0; f < nFluid_; f++) {
         for (int s = 0; s < Q; s++) {
            int dir = push_ ? s : lattice_.getOpp(s);
            int nbr[3];
            bool inside = true;
            for (int d = 0; d < 3; d++) {
               nbr[d] = fluidPts_[f][d] + lattice_.getVel(dir, d);
               if (periodic_[d]) {
                  if (nbr[d] < 0) nbr[d] += dims_[d];
                  else if (nbr[d] >= dims_[d]) nbr[d] -= dims_[d];
               }
               if (nbr[d] < 0 || nbr[d] >= dims_[d]) inside = false;
            }
            int nbrFluid = inside ? grid_[getGridIdx(nbr[0], nbr[1], nbr[2])] : -1;
            if (nbrFluid < 0) {
               adjacency_[(size_t)nFluid_ * s + f] = nFluid_ * lattice_.getOpp(s) + f;
            } else {
               adjacency_[(size_t)nFluid_ * s + f] = nFluid_ * s + nbrFluid;
            }
         }
      }
   }

   size_t denseIndex(int f) const
   {
      return (size_t)fluidPts_[f][0] +
             (size_t)dims_[0] * ((size_t)fluidPts_[f][1] + (size_t)dims_[1] * fluidPts_[f][2]);
   }

private:
   bool push_;
   int dims_[3];
   int periodic_[3];
};

struct ExposedAA : public PropagationAA {
   using PropagationAA::PropagationAA;
   Pdf* raw() { return dstrb_; }
};

struct ExposedAB : public PropagationAB {
   using PropagationAB::PropagationAB;
   Pdf* raw() { return dstrb_; }
};

struct AppState {
   Parameters* parameters = nullptr;
   Lattice* lattice = nullptr;
   GeometryAAAB* geometry = nullptr;
   Communication* comm = nullptr;
   ExposedAA* aa = nullptr;
   ExposedAB* ab = nullptr;
};

AppState g_app;

void app_release()
{
   delete g_app.aa;
   delete g_app.ab;
   delete g_app.comm;
   delete g_app.geometry;
   delete g_app.lattice;
   delete g_app.parameters;
   g_app = AppState();
}

}  // namespace

extern "C" {

int ref_lattice_size(void) { return _LATTICESIZE_; }

/*
 * variant: 0 AA Base, 1 AA Unroll (Q19), 2 AB push Base, 3 AB push Unroll (Q19),
 *          4 AB pull Base, 5 AB pull Unroll (Q19).
 * f_init : logical populations, dense [q][z][y][x]; direction s of each cell.
 *          Placed with the reference's conventions: AA stores direction s in
 *          slot opp(s) (src/propagation/PropagationAA.cpp:104-116); AB stores
 *          slot s in both buffers (src/propagation/PropagationAB.cpp:130-143).
 * f_raw  : final contents of the population buffer the reference reads back
 *          (AA: the single buffer; AB: dstrb_ after the last swap), dense
 *          [q][z][y][x]; NaN at solid cells.
 * Returns 0 on success, nonzero for an unsupported variant.
 */
int ref_box_run(int variant, int nx, int ny, int nz, const unsigned char* solid,
                const int* periodic, double omega, double gx, const double* f_init,
                int nsteps, double* f_raw, double* seconds)
{
   const int Q = _LATTICESIZE_;
   if (variant < 0 || variant > 5) return 1;
   if ((variant & 1) && Q != 19) return 2;
   lbm_ref_omega = omega;
   lbm_ref_gravity = gx;

   Parameters parameters;
   Lattice* lattice = make_lattice();
   bool aa = variant <= 1;
   bool push = (variant == 2 || variant == 3);
   HarnessGeometry geometry(*lattice, parameters, nx, ny, nz, solid, periodic, push);
   geometry.setupAdjacency();
   const int nFluid = geometry.getNumFluidPts();
   const size_t ncell = (size_t)nx * ny * nz;

   std::vector<Pdf> a((size_t)nFluid * Q, 0.0), b((size_t)nFluid * Q, 0.0);
   for (int f = 0; f < nFluid; f++) {
      size_t dense = geometry.denseIndex(f);
      for (int s = 0; s < Q; s++) {
         double v = f_init[(size_t)s * ncell + dense];
         if (aa) {
            a[(size_t)nFluid * lattice->getOpp(s) + f] = v;
         } else {
            a[(size_t)nFluid * s + f] = v;
            b[(size_t)nFluid * s + f] = v;
         }
      }
   }

   Pdf* src = a.data();
   Pdf* tgt = b.data();
   auto t0 = std::chrono::steady_clock::now();
   if (aa) {
      KernelAA* k = (variant == 1) ? (KernelAA*)new KernelAA_SOA_Unroll(*lattice, geometry)
                                   : (KernelAA*)new KernelAA_SOA_Base(*lattice, geometry);
      k->setup();
      for (int t = 0; t < nsteps; t++) {
         if (t % 2 == 0) k->timestepEvenForce(src, 0, nFluid);
         else k->timestepOddForce(src, 0, nFluid);
      }
      delete k;
   } else {
      KernelAB* k = nullptr;
      switch (variant) {
         case 2: k = new KernelAB_SOA_Base(*lattice, geometry); break;
         case 3: k = new KernelAB_SOA_Unroll(*lattice, geometry); break;
         case 4: k = new KernelAB_SOA_Pull(*lattice, geometry); break;
         default: k = new KernelAB_SOA_Unroll_Pull(*lattice, geometry); break;
      }
      k->setup();
      for (int t = 0; t < nsteps; t++) {
         k->timestepForce(src, tgt, 0, nFluid);
         std::swap(src, tgt);
      }
      delete k;
   }
   auto t1 = std::chrono::steady_clock::now();
   if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();

   const double nan = std::numeric_limits<double>::quiet_NaN();
   for (size_t i = 0; i < (size_t)Q * ncell; i++) f_raw[i] = nan;
   for (int f = 0; f < nFluid; f++) {
      size_t dense = geometry.denseIndex(f);
      for (int s = 0; s < Q; s++) f_raw[(size_t)s * ncell + dense] = src[(size_t)nFluid * s + f];
   }
   delete[] geometry.adjacency_;
   delete lattice;
   return 0;
}

/*
 * Reference app flow, part 1: read the input file and build the cylinder
 * exactly as src/Main.cpp:45-74 does.  dims = (Lx, Ly, Lz), x the pipe axis.
 * omega / gx set the run-time stand-ins for _OMEGA_ / _GRAVITY_.
 */
int ref_app_prepare(const char* input_file, double omega, double gx, int* dims,
                    long long* nfluid, int* steps, int* prop_pattern)
{
   app_release();
   lbm_ref_omega = omega;
   lbm_ref_gravity = gx;
   g_app.parameters = new Parameters;
   g_app.parameters->readInput(std::string(input_file));
   g_app.lattice = make_lattice();
   g_app.geometry = new GeometryAAAB(*g_app.lattice, *g_app.parameters);
   g_app.geometry->decomposeDomain();
   g_app.geometry->setupGrid();
   g_app.geometry->setup();
   g_app.geometry->assignFluidIndices();
   g_app.geometry->setupAdjacency();
   g_app.comm = new Communication(*g_app.lattice, *g_app.geometry, *g_app.parameters);
   g_app.comm->kokkosSyclNoNeighborSetup();
   for (int d = 0; d < 3; d++) dims[d] = g_app.geometry->getTotalLengthByDim(d);
   *nfluid = g_app.geometry->getGlobalNumFluidPts();
   *steps = g_app.parameters->getTimesteps();
   *prop_pattern = g_app.parameters->getPropPattern();
   return 0;
}

/*
 * Part 2: PropagationAA/AB setup + run (src/Main.cpp:84-126), then the
 * reference readouts: rho via getRho, u via getVelocity (no F/2 shift) at the
 * step index the reference's own checkResult uses, and the raw population
 * buffer.  Arrays are dense over (Lx, Ly, Lz), x fastest (u and f_raw planar:
 * [component][cell]); NaN at walls.
 */
int ref_app_execute(double* rho, double* u, double* f_raw, double* seconds)
{
   if (!g_app.geometry) return 1;
   Geometry& g = *g_app.geometry;
   const int Q = _LATTICESIZE_;
   const int L0 = g.getTotalLengthByDim(0), L1 = g.getTotalLengthByDim(1),
             L2 = g.getTotalLengthByDim(2);
   const size_t ncell = (size_t)L0 * L1 * L2;
   const int steps = g_app.parameters->getTimesteps();
   Propagation* prop = nullptr;
   Pdf* raw = nullptr;
   int readStep = steps;
   auto t0 = std::chrono::steady_clock::now();
   if (g_app.parameters->getPropPattern() == 1) {
      g_app.aa = new ExposedAA(*g_app.lattice, g, *g_app.comm, *g_app.parameters);
      g_app.aa->setup();
      g_app.aa->run();
      prop = g_app.aa;
      raw = g_app.aa->raw();
   } else {
      g_app.ab = new ExposedAB(*g_app.lattice, g, *g_app.comm, *g_app.parameters);
      g_app.ab->setup();
      g_app.ab->run();
      prop = g_app.ab;
      raw = g_app.ab->raw();
      readStep = steps - 1;
   }
   auto t1 = std::chrono::steady_clock::now();
   if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();

   const double nan = std::numeric_limits<double>::quiet_NaN();
   for (size_t i = 0; i < ncell; i++) {
      rho[i] = nan;
      u[i] = u[ncell + i] = u[2 * ncell + i] = nan;
   }
   for (size_t i = 0; i < (size_t)Q * ncell; i++) f_raw[i] = nan;
   const int nFluid = g.getNumFluidPts();
   for (int f = 0; f < nFluid; f++) {
      const std::vector<int>& p = g.fluidPts_[f];
      size_t dense = (size_t)p[0] + (size_t)L0 * ((size_t)p[1] + (size_t)L1 * p[2]);
      rho[dense] = prop->getRho(f, readStep);
      std::vector<Pdf> v = prop->getVelocity(f, readStep);
      for (int d = 0; d < 3; d++) u[(size_t)d * ncell + dense] = v[d];
      for (int s = 0; s < Q; s++) f_raw[(size_t)s * ncell + dense] = raw[(size_t)nFluid * s + f];
   }
   app_release();
   return 0;
}

/*
 * Part 2, compact form: the same run, returning the reference's own buffers
 * in its own layout instead of dense arrays -- the raw population buffer
 * before the run (raw_init, the rest state PropagationAA/AB::initialize
 * wrote) and after it (raw_final), both [Q][nFluid]; the adjacency list of
 * GeometryAAAB::setupAdjacency, [Q][nFluid]; the fluid points in the
 * reference's sorted order, [nFluid][3] as (i, j, k).
 */
int ref_app_execute_compact(double* raw_init, double* raw_final, int* adjacency, int* fluid_pts,
                            double* seconds)
{
   if (!g_app.geometry) return 1;
   Geometry& g = *g_app.geometry;
   const int Q = _LATTICESIZE_;
   const int nFluid = g.getNumFluidPts();
   for (size_t k = 0; k < (size_t)Q * nFluid; k++) adjacency[k] = g.adjacency_[k];
   for (int f = 0; f < nFluid; f++)
      for (int d = 0; d < 3; d++) fluid_pts[3 * f + d] = g.fluidPts_[f][d];
   Pdf* raw = nullptr;
   auto t0 = std::chrono::steady_clock::now();
   if (g_app.parameters->getPropPattern() == 1) {
      g_app.aa = new ExposedAA(*g_app.lattice, g, *g_app.comm, *g_app.parameters);
      g_app.aa->setup();
      g_app.aa->initialize();
      for (size_t k = 0; k < (size_t)Q * nFluid; k++) raw_init[k] = g_app.aa->raw()[k];
      g_app.aa->run();
      raw = g_app.aa->raw();
   } else {
      g_app.ab = new ExposedAB(*g_app.lattice, g, *g_app.comm, *g_app.parameters);
      g_app.ab->setup();
      g_app.ab->initialize();
      for (size_t k = 0; k < (size_t)Q * nFluid; k++) raw_init[k] = g_app.ab->raw()[k];
      g_app.ab->run();
      raw = g_app.ab->raw();
   }
   auto t1 = std::chrono::steady_clock::now();
   if (seconds) *seconds = std::chrono::duration<double>(t1 - t0).count();
   for (size_t k = 0; k < (size_t)Q * nFluid; k++) raw_final[k] = raw[k];
   app_release();
   return 0;
}

}  // extern "C"
