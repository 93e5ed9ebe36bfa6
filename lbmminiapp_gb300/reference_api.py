"""The reference's host-side interface over the GB300 library.

Mirrors lbmminiapp's ``Parameters`` (src/Parameters.cpp:20-92) and
``PropagationAA`` / ``PropagationAB`` (src/propagation/PropagationAA.cpp:10-327,
src/propagation/PropagationAB.cpp:16-281, src/propagation/Propagation.cpp:164-212):
same input-file keys, same method names, same printed lines, so a run of the
reference's ``test/*.txt`` files reads the same.  The geometry is the
reference's cylinder (src/geometries/Geometry.cpp:59-71,112-140), periodic in x
only as on one rank (src/geometries/GeometryAAAB.cpp:56-66).

Keys beyond the reference's (ignored by it, so its input files stay valid):
``lattice 19|27``, ``omega`` or ``tau`` (the reference's compile-time _OMEGA_,
default 1.0), ``gravity`` (its _GRAVITY_, default 1e-6), ``storage
f64|f32|bf16|f16``, ``arithmetic auto|f64|f64x``.
"""
from __future__ import annotations

import time

import numpy as np

from .simulation import Simulation, cylinder

_ONETHIRD = 0.333333333333333333  # src/Parameters.hh:33


class Parameters:
    """Input-file reader with the reference's keys and defaults
    (src/Parameters.cpp:23-30, :50-77).  Unknown keys are ignored."""

    def __init__(self):
        self.densityChange = 0.01
        self.geometryLibID = 1
        self.propPattern = 0
        self.pullSetting = 0
        self.unrollSetting = 0
        self.simulationSize = 1.0
        self.timesteps = 1
        self.writeVtk = 0
        self.lattice = 19
        self.omega = 1.0
        self.gravity = 0.000001
        self.storage = "f64"
        self.arithmetic = "auto"
        self.echo = []

    def readInput(self, input_file):
        keys = {
            "densitychange": ("densityChange", float), "densityChange": ("densityChange", float),
            "proppattern": ("propPattern", int), "propPattern": ("propPattern", int),
            "pull": ("pullSetting", int), "unroll": ("unrollSetting", int),
            "simulationsize": ("simulationSize", float), "simulationSize": ("simulationSize", float),
            "timesteps": ("timesteps", int), "writevtk": ("writeVtk", int),
            "lattice": ("lattice", int), "omega": ("omega", float), "gravity": ("gravity", float),
            "storage": ("storage", str), "arithmetic": ("arithmetic", str),
        }
        with open(input_file) as fh:
            for line in fh:
                self.echo.append(line.rstrip("\n"))
                parts = line.split()
                if len(parts) < 2:
                    continue
                if parts[0] == "tau":
                    self.omega = 1.0 / float(parts[1])
                elif parts[0] in keys:
                    attr, conv = keys[parts[0]]
                    if conv is int:  # atoi: integer part
                        setattr(self, attr, int(float(parts[1])))
                    else:
                        setattr(self, attr, conv(parts[1]))
        return self

    # getters with the reference's names (src/Parameters.hh:53-60)
    def getPropPattern(self):
        return self.propPattern

    def getPullSetting(self):
        return self.pullSetting

    def getUnrollSetting(self):
        return self.unrollSetting

    def getSimulationSize(self):
        return self.simulationSize

    def getTimesteps(self):
        return self.timesteps


class Propagation:
    """Common part of PropagationAA / PropagationAB over one library handle."""

    pattern = "aa"

    def __init__(self, parameters: Parameters, device=0, out=print):
        self.parameters = parameters
        self.device = device
        self.out = out
        self.sim = None
        self.dims = None
        self.solid = None
        self.elapsed = None

    def setup(self):
        p = self.parameters
        self.dims, self.solid = cylinder(p.simulationSize)
        nx, ny, nz = self.dims
        pattern = self.pattern if self.pattern == "aa" else ("ab_pull" if p.pullSetting == 1 else "ab_push")
        self.sim = Simulation(nx, ny, nz, lattice=p.lattice, pattern=pattern, omega=p.omega,
                              force=(p.gravity, 0.0, 0.0), periodic=(1, 0, 0), storage=p.storage,
                              arithmetic=p.arithmetic, unroll=bool(p.unrollSetting), device=self.device)
        self.sim.set_solid(self.solid)
        self.out(f"Simulation has {self.sim.nfluid} fluid points")

    def initialize(self):
        self.sim.init_equilibrium()  # rest state f = w (PropagationAA.cpp:104-116)

    def run(self):
        self.initialize()
        steps = self.parameters.timesteps
        self.sim.synchronize()
        t0 = time.perf_counter()
        self.sim.step(steps)
        self.sim.synchronize()
        self.elapsed = time.perf_counter() - t0
        self.printMFLUPS(self.elapsed)
        self.rho, self.u = self.sim.macros()
        read_step = steps if self.pattern == "aa" else steps - 1
        ok = self.checkResult(read_step)
        if self.parameters.writeVtk:
            self.writeVTK(read_step)
        return ok

    def writeVTK(self, currentStep, path="outs.00000.vtk"):
        """src/propagation/Propagation.cpp:36-161 (single rank: outs.00000.vtk
        in the working directory), from the readouts of the last run."""
        from .vtk import write_vtk
        write_vtk(path, self.rho, self.u, self.solid)
        return path

    def getRho(self, i, j, k):
        return float(self.rho[k, j, i])

    def getVelocity(self, i, j, k):
        return [float(self.u[d, k, j, i]) for d in range(3)]

    def checkResult(self, currentStep):
        """Centre-line Hagen-Poiseuille check (src/propagation/Propagation.cpp:164-197):
        passes when (u_x - u_expected) / u_expected < 0.25."""
        nx, ny, nz = self.dims
        ci, cj, ck = (nx - 1) // 2, (ny - 1) // 2, (nz - 1) // 2
        if self.solid[ck, cj, ci]:
            return None
        diameter = 16.0 * self.parameters.simulationSize
        nu = _ONETHIRD * (1.0 / self.parameters.omega - 0.5)
        rho = self.getRho(ci, cj, ck)
        vel = self.getVelocity(ci, cj, ck)[0]
        expected = (self.parameters.gravity * diameter * diameter) / (16.0 * rho * nu)
        ok = (vel - expected) / expected < 0.25
        self.out("Passed baseline validation" if ok else "Failed baseline validation")
        self.centre_velocity = vel
        return ok

    def printMFLUPS(self, runtime):
        """src/propagation/Propagation.cpp:200-212."""
        mflups = (self.sim.nfluid * self.parameters.timesteps) / (1000000 * runtime)
        mfeups = mflups * (self.parameters.lattice - 1)
        self.out("Overall performance")
        self.out(f"Total {mfeups:g} MFEUPS (million fluid elementary updates per second)")
        self.out(f"Total {mflups:g} MFLUPS (million fluid lattice updates per second)")
        self.out(f"Avg {mflups:g} MFLUPS per rank")
        self.mflups = mflups
        return mflups

    def close(self):
        if self.sim:
            self.sim.close()
            self.sim = None


class PropagationAA(Propagation):
    pattern = "aa"


class PropagationAB(Propagation):
    pattern = "ab"


def main(input_file, device=0, out=print):
    """src/Main.cpp:22-145 on one GPU: parameters, propagation by propPattern,
    setup, run.  Returns the propagation object (closed)."""
    out("Run started on 1 tasks")
    t0 = time.perf_counter()
    p = Parameters().readInput(input_file)
    for line in p.echo:
        out(line)
    prop = (PropagationAA if p.propPattern == 1 else PropagationAB)(p, device=device, out=out)
    prop.setup()
    prop.run()
    prop.close()
    out(f"Total runtime (rank 0): {time.perf_counter() - t0}")
    return prop


if __name__ == "__main__":
    import sys
    main(sys.argv[1])
