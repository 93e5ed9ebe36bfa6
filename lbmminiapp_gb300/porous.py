"""Flow through a periodic sphere packing: permeability from the forward run
and the adjoint of the mean flux with respect to the per-cell porosity.

Workload: a periodic n^3 box, seeded non-overlapping solid spheres
(``workloads.sphere_packing``) with half-way bounce-back on their surfaces, a
uniform body force g_x, BGK with relaxation time tau, started from rest.

* Permeability after ``steps`` steps: k = nu <u_x> / g_x with
  nu = (tau - 1/2) / 3 and <u_x> the mean over all cells (solid cells count as
  u = 0) of the force-shifted velocity u = (sum c f + F/2) / rho.
* Mean-flux gradient: L = <u_x> at the last step, differentiated with respect
  to a per-cell partial bounce-back fraction s(x) at s = 0 through the
  checkpointed AB-push adjoint (``adjoint.Rollout``).  AA and AB-push storage
  hold the same populations after every step (the collision is the same
  function of the same values), so this is also the gradient of the AA run.

The reduced-precision results (FP16 or BF16 shifted storage with FP32
collision, FP32 adjoint) are compared with the FP64 forward and the FP64
adjoint on the same packing.
"""
from __future__ import annotations

import time

import numpy as np

from .simulation import Simulation
from . import workloads


def viscosity(tau):
    return (tau - 0.5) / 3.0


def mean_velocity_x(sim: Simulation, gx: float) -> float:
    """<u_x> over all cells, u = (sum c f + F/2) / rho, u = 0 in solid cells."""
    rho, u = sim.macros()
    fluid = np.isfinite(rho)
    ux = np.where(fluid, u[0] + 0.5 * gx / np.where(fluid, rho, 1.0), 0.0)
    return float(ux.sum() / ux.size)


def packing(n, solid_fraction=0.35, rmin=6.0, rmax=12.0, seed=0):
    solid, _, radii = workloads.sphere_packing(n, solid_fraction, rmin, rmax, seed=seed)
    return solid, len(radii)


def forward(solid, tau, gx, steps, lattice=27, pattern="aa", storage="f16", arithmetic="auto", device=0,
            compact=None):
    """Run ``steps`` steps from rest; returns a dict with the permeability, the
    mean velocity, the wall time of the steps and the fluid-cell update rate
    (MFLUP/s).  compact: compact fluid-only storage (default: for AA with
    shifted storage, the only case that has it)."""
    nz, ny, nx = solid.shape
    if compact is None:
        compact = pattern == "aa" and storage != "f64"
    with Simulation(nx, ny, nz, lattice=lattice, pattern=pattern, omega=1.0 / tau, force=(gx, 0.0, 0.0),
                    periodic=(1, 1, 1), storage=storage, arithmetic=arithmetic, device=device,
                    compact=compact) as sim:
        sim.set_solid(solid)
        sim.init_equilibrium()
        sim.synchronize()
        t0 = time.perf_counter()
        sim.step(steps)
        sim.synchronize()
        dt = time.perf_counter() - t0
        ux = mean_velocity_x(sim, gx)
        return {"storage": storage, "arithmetic": arithmetic, "pattern": pattern, "steps": steps,
                "mean_ux": ux, "permeability": viscosity(tau) * ux / gx, "seconds": dt,
                "mflups": sim.nfluid * steps / dt / 1e6}


def flux_weight(solid):
    """Loss weight W for L = <u_x>: 1/ncell on the x component of fluid cells."""
    w = np.zeros((3,) + solid.shape)
    w[0] = (~solid.astype(bool)) / solid.size
    return w


def flux_gradient(solid, tau, gx, steps, checkpoint_every, storage="f16", adjoint="f32", lattice=27, device=0,
                  arithmetic="auto"):
    """dL/ds(x) of L = <u_x> after ``steps`` steps (s = per-cell porosity, at
    s = 0).  Returns (loss, gradient (nz, ny, nx) float64 numpy, seconds of
    forward + reverse sweep).  ``arithmetic`` is the forward's collision
    arithmetic ("auto": F64X for FP64 storage, FP32 otherwise)."""
    import gc

    import torch
    from .adjoint import Rollout

    nz, ny, nx = solid.shape
    sim = Simulation(nx, ny, nz, lattice=lattice, pattern="ab_push", omega=1.0 / tau, force=(gx, 0.0, 0.0),
                     periodic=(1, 1, 1), storage=storage, arithmetic=arithmetic, device=device)
    r = None
    try:
        sim.set_solid(solid)
        sim.init_equilibrium()
        r = Rollout(sim, steps, checkpoint_every, "velocity", flux_weight(solid), (steps, steps), adjoint=adjoint)
        t0 = time.perf_counter()
        loss = r.run_forward(store=True)
        _, gS = r.run_backward(grad_force=False)
        torch.cuda.synchronize(device)
        dt = time.perf_counter() - t0
        grad = r.from_plane(gS).cpu().numpy()
        return loss, grad, dt
    finally:
        if r is not None:
            r.release()
        del r
        sim.close()
        gc.collect()
        torch.cuda.empty_cache()


def gradient_errors(g, g_ref, fluid):
    """Relative L2 and max-norm errors of g against g_ref over fluid cells,
    and their correlation."""
    a, b = g[fluid], g_ref[fluid]
    d = a - b
    return {"rel_l2": float(np.linalg.norm(d) / np.linalg.norm(b)),
            "rel_max": float(np.abs(d).max() / np.abs(b).max()),
            "corr": float(np.corrcoef(a, b)[0, 1])}
