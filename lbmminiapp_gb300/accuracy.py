"""Error of the shifted FP32 / BF16 / FP16 storage against FP64 storage on the
Taylor-Green + noise workload (D3Q19 AA, periodic box, tau = 0.55).

For each storage the same initial state runs `steps` lattice steps; density,
velocity and total mass are compared with the FP64-storage run (F64X
arithmetic, itself within 1e-10 of the reference):

* u_rel_l2   ||u - u_64||_2 / ||u_64||_2 over all cells
* u_rel_max  max |u - u_64| / max |u_64|
* rho_max    max |rho - rho_64|
* mass_rel   (M - M_64) / M_64 with M the FP64 sum of rho (conserved sums)
"""
from __future__ import annotations

import numpy as np

from .simulation import Simulation
from .workloads import taylor_green


def error_table(n=512, steps=1000, tau=0.55, storages=("f32", "bf16", "f16"), U=0.05, noise=1e-3, seed=2024,
                lattice=19, device=0):
    u0 = taylor_green(n, n, n, U=U, noise=noise, seed=seed)

    def run(storage):
        sim = Simulation(n, n, n, lattice=lattice, pattern="aa", omega=1.0 / tau, force=(0, 0, 0), storage=storage,
                         arithmetic="auto", device=device)
        sim.init_equilibrium(None, u0)
        m0 = sim.conserved()[0]
        sim.step(steps)
        rho, u = sim.macros()
        m1 = sim.conserved()[0]
        sim.close()
        return rho, u, m0, m1

    rho64, u64, m0_64, m1_64 = run("f64")
    table = {"f64": {"mass_drift_rel": float((m1_64 - m0_64) / m0_64)}}
    nu = np.sqrt(np.sum(u64 * u64))
    umax = np.abs(u64).max()
    for st in storages:
        rho, u, m0, m1 = run(st)
        du = u - u64
        table[st] = {
            "u_rel_l2": float(np.sqrt(np.sum(du * du)) / nu),
            "u_rel_max": float(np.abs(du).max() / umax),
            "rho_max": float(np.abs(rho - rho64).max()),
            "mass_rel": float((m1 - m1_64) / m1_64),
            "mass_drift_rel": float((m1 - m0) / m0),
        }
        del rho, u, du
    return table
