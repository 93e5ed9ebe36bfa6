// lbm-gb300-app: the reference's single-rank driver flow (src/Main.cpp:22-145)
// over the GB300 library's C ABI.
//
//   lbm-gb300-app <inputfile>
//
// Reads the reference's input files (keys of src/Parameters.cpp:50-77, plus
// lattice / omega / tau / gravity / storage / arithmetic, which the reference
// ignores), builds its cylinder (src/geometries/Geometry.cpp:59-71,112-140,
// periodic in x only as on one rank), runs AA or AB push / pull, and prints
// the reference's lines: the input echo, fluid-point count, MFEUPS / MFLUPS
// (src/propagation/Propagation.cpp:200-212) and the centre-line Poiseuille
// check (src/propagation/Propagation.cpp:164-197); with "writevtk 1" it
// writes outs.00000.vtk like the reference.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/lbm_gb300.h"

namespace {

struct Params {
   double densityChange = 0.01;
   int propPattern = 0;   // AB = 0, AA = 1
   int pull = 0;
   int unroll = 0;
   double simulationSize = 1.0;
   int timesteps = 1;
   int writeVtk = 0;
   int lattice = 19;
   double omega = 1.0;          // the reference's _OMEGA_ default
   double gravity = 0.000001;   // the reference's _GRAVITY_
   int storage = LBM_STORE_F64;
   int arithmetic = LBM_ARITH_AUTO;
};

bool read_input(const char* path, Params& p)
{
   std::ifstream in(path);
   if (!in) return false;
   std::string line;
   while (std::getline(in, line)) {
      std::cout << line << std::endl;
      std::istringstream iss(line);
      std::string key, val;
      if (!(iss >> key >> val)) continue;
      if (key == "densitychange" || key == "densityChange") p.densityChange = std::atof(val.c_str());
      else if (key == "proppattern" || key == "propPattern") p.propPattern = std::atoi(val.c_str());
      else if (key == "pull") p.pull = std::atoi(val.c_str());
      else if (key == "unroll") p.unroll = std::atoi(val.c_str());
      else if (key == "simulationsize" || key == "simulationSize") p.simulationSize = std::atof(val.c_str());
      else if (key == "timesteps") p.timesteps = std::atoi(val.c_str());
      else if (key == "writevtk") p.writeVtk = std::atoi(val.c_str());
      else if (key == "lattice") p.lattice = std::atoi(val.c_str());
      else if (key == "omega") p.omega = std::atof(val.c_str());
      else if (key == "tau") p.omega = 1.0 / std::atof(val.c_str());
      else if (key == "gravity") p.gravity = std::atof(val.c_str());
      else if (key == "storage")
         p.storage = val == "f32" ? LBM_STORE_F32 : val == "bf16" ? LBM_STORE_BF16 : val == "f16" ? LBM_STORE_F16
                                                                                                    : LBM_STORE_F64;
      else if (key == "arithmetic")
         p.arithmetic = val == "f64" ? LBM_ARITH_F64 : val == "f64x" ? LBM_ARITH_F64X : LBM_ARITH_AUTO;
   }
   return true;
}

// Propagation::writeVTK (src/propagation/Propagation.cpp:36-161) on one rank:
// outs.00000.vtk with rho, point id, velocity and node coordinates, x fastest,
// default stream formatting.  Non-fluid points: rho 0, velocity 0 0 0, id
// LAT_PT_WALL (-10); fluid points are numbered in x-fastest order.
bool write_vtk(const char* path, const int dims[3], const std::vector<uint8_t>& solid,
               const std::vector<double>& rho, const std::vector<double>& u)
{
   std::ofstream f(path);
   if (!f) return false;
   const size_t n = solid.size();
   f << "# vtk DataFile Version 3.0" << "\n" << "Placeholder" << "\n" << "ASCII" << "\n"
     << "DATASET STRUCTURED_POINTS" << "\n"
     << "DIMENSIONS " << dims[0] << " " << dims[1] << " " << dims[2] << "\n"
     << "ORIGIN 0 0 0" << "\n" << "SPACING 1 1 1" << "\n" << "POINT_DATA " << n << "\n";
   f << "SCALARS rho double" << "\n" << "LOOKUP_TABLE default" << "\n";
   for (size_t c = 0; c < n; c++) f << (solid[c] ? 0.0 : rho[c]) << "\n";
   f << "SCALARS id int" << "\n" << "LOOKUP_TABLE default" << "\n";
   long long fid = 0;
   for (size_t c = 0; c < n; c++) f << (solid[c] ? -10LL : fid++) << "\n";
   f << "VECTORS velocity double" << "\n";
   for (size_t c = 0; c < n; c++) {
      if (solid[c]) f << 0.0 << " " << 0.0 << " " << 0.0 << "\n";
      else f << u[c] << " " << u[n + c] << " " << u[2 * n + c] << "\n";
   }
   f << "VECTORS nodes int" << "\n";
   for (int k = 0; k < dims[2]; k++)
      for (int j = 0; j < dims[1]; j++)
         for (int i = 0; i < dims[0]; i++) f << i << " " << j << " " << k << "\n";
   return (bool)f;
}

int die(lbm_handle* h, lbm_status s, const char* what)
{
   std::fprintf(stderr, "%s failed: %s (%s)\n", what, lbm_status_string(s), h ? lbm_last_error(h) : "");
   if (h) lbm_destroy(h);
   return 1;
}

}  // namespace

int main(int argc, char** argv)
{
   if (argc < 2) {
      std::fprintf(stderr, "usage: %s <inputfile>\n", argv[0]);
      return 2;
   }
   std::cout << "Run started on 1 tasks" << std::endl;
   const auto tStart = std::chrono::steady_clock::now();
   Params p;
   if (!read_input(argv[1], p)) {
      std::fprintf(stderr, "cannot read %s\n", argv[1]);
      return 2;
   }

   int dims[3];
   lbm_status s = lbm_geometry_cylinder(p.simulationSize, dims, nullptr);
   if (s != LBM_OK) return die(nullptr, s, "lbm_geometry_cylinder");
   std::vector<uint8_t> solid((size_t)dims[0] * dims[1] * dims[2]);
   lbm_geometry_cylinder(p.simulationSize, dims, solid.data());

   lbm_config cfg;
   lbm_config_default(&cfg);
   cfg.lattice = p.lattice;
   cfg.prop_pattern = p.propPattern == 1 ? LBM_PATTERN_AA : LBM_PATTERN_AB;
   cfg.pull = p.pull;
   cfg.unroll = p.unroll;
   cfg.nx = dims[0];
   cfg.ny = dims[1];
   cfg.nz = dims[2];
   cfg.periodic[0] = 1;
   cfg.periodic[1] = 0;
   cfg.periodic[2] = 0;
   cfg.omega = p.omega;
   cfg.force[0] = p.gravity;
   cfg.force[1] = cfg.force[2] = 0.0;
   cfg.storage = p.storage;
   cfg.arithmetic = p.arithmetic;
   lbm_handle* h = nullptr;
   if ((s = lbm_create(&cfg, &h)) != LBM_OK) return die(nullptr, s, "lbm_create");
   if ((s = lbm_set_solid(h, solid.data())) != LBM_OK) return die(h, s, "lbm_set_solid");
   lbm_info info;
   lbm_get_info(h, &info);
   std::cout << "Simulation has " << info.nfluid << " fluid points" << std::endl;

   // initialize + run (PropagationAA.cpp:126-215 / PropagationAB.cpp:155-219)
   if ((s = lbm_init_equilibrium(h, nullptr, nullptr)) != LBM_OK) return die(h, s, "lbm_init_equilibrium");
   lbm_synchronize(h);
   const auto t0 = std::chrono::steady_clock::now();
   if ((s = lbm_step(h, p.timesteps)) != LBM_OK) return die(h, s, "lbm_step");
   if ((s = lbm_synchronize(h)) != LBM_OK) return die(h, s, "lbm_synchronize");
   const double runtime = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();

   const double mflups = ((double)info.nfluid * p.timesteps) / (1000000 * runtime);
   const double mfeups = mflups * (p.lattice - 1);
   std::cout << "Overall performance" << std::endl;
   std::cout << "Total " << mfeups << " MFEUPS (million fluid elementary updates per second)" << std::endl;
   std::cout << "Total " << mflups << " MFLUPS (million fluid lattice updates per second)" << std::endl;
   std::cout << "Avg " << mflups << " MFLUPS per rank" << std::endl;

   // checkResult: centre-line velocity against Hagen-Poiseuille
   const size_t n = solid.size();
   std::vector<double> rho(n), u(3 * n);
   if ((s = lbm_get_macros(h, rho.data(), u.data())) != LBM_OK) return die(h, s, "lbm_get_macros");
   const int ci = (dims[0] - 1) / 2, cj = (dims[1] - 1) / 2, ck = (dims[2] - 1) / 2;
   const size_t c = (size_t)ci + (size_t)dims[0] * ((size_t)cj + (size_t)dims[1] * ck);
   if (!solid[c]) {
      const double diameter = 16.0 * p.simulationSize;
      const double nu = 0.333333333333333333 * (1.0 / p.omega - 0.5);
      const double expected = (p.gravity * diameter * diameter) / (16.0 * rho[c] * nu);
      const double vel = u[c];
      std::cout << ((vel - expected) / expected < 0.25 ? "Passed baseline validation" : "Failed baseline validation")
                << std::endl;
      std::printf("Centre-line velocity %.17g (Poiseuille %.17g)\n", vel, expected);
      std::fflush(stdout);
   }
   if (p.writeVtk && !write_vtk("outs.00000.vtk", dims, solid, rho, u)) {
      std::fprintf(stderr, "cannot write outs.00000.vtk\n");
      lbm_destroy(h);
      return 1;
   }
   lbm_destroy(h);
   const double total = std::chrono::duration<double>(std::chrono::steady_clock::now() - tStart).count();
   std::cout << "Total runtime (rank 0): " << total << std::endl;
   return 0;
}
