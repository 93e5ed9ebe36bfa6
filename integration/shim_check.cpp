// Builds every reference-side shim against the unmodified reference headers and
// drives them through the reference's own set-up flow (src/Main.cpp:45-126):
// Parameters from an input file, the GeometryAAAB cylinder, Communication, then
// PropagationGB300 and the compact kernel shims.  gb300_shim_check returns the
// number of stages passed (1 PropagationGB300::setup, 2 compact kernel shims
// constructed, 3 the propagation run with its MFLUPS and validation lines) and
// leaves the first failure's message in msg; with no GPU the library's status
// comes back through the shims' exception at stage 0.
#include <cstdio>
#include <exception>

#include "Communication.hh"
#include "GeometryAAAB.hh"
#include "KernelGB300Compact.hh"
#include "KernelGB300Dense.hh"
#include "LatticeD3Q19.hh"
#include "LatticeD3Q27.hh"
#include "Parameters.hh"
#include "PropagationGB300.hh"

extern "C" int gb300_shim_check(const char* input_file, char* msg, int msglen)
{
   Parameters parameters;
   parameters.readInput(std::string(input_file));
   Lattice* lattice = nullptr;
   if (_LATTICESIZE_ == 27) lattice = new LatticeD3Q27;
   else lattice = new LatticeD3Q19;
   GeometryAAAB geometry(*lattice, parameters);
   geometry.decomposeDomain();
   geometry.setupGrid();
   geometry.setup();
   geometry.assignFluidIndices();
   geometry.setupAdjacency();
   Communication comm(*lattice, geometry, parameters);
   comm.kokkosSyclNoNeighborSetup();
   int stage = 0;
   msg[0] = '\0';
   try {
      PropagationGB300 prop(*lattice, geometry, comm, parameters);
      prop.setup();
      stage = 1;
      if (parameters.getPropPattern() == 1) {
         KernelAA_GB300Compact k(*lattice, geometry, parameters);
         KernelAA_GB300 d(*lattice, geometry, prop.handle());
         k.setup();
         d.setup();
      } else {
         KernelAB_GB300Compact k(*lattice, geometry, parameters);
         KernelAB_GB300 d(*lattice, geometry, prop.handle());
         k.setup();
         d.setup();
      }
      stage = 2;
      prop.run();
      stage = 3;
   } catch (const std::exception& e) {
      snprintf(msg, (size_t)msglen, "%s", e.what());
   }
   delete lattice;
   return stage;
}
