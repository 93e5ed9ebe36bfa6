"""F64X cells that leave the fast path's range (a population at or above
1/4, a negative one, a fast flow) take the exact FP64 collision inside the
pipelined kernel, which reads the cell's inputs again from shared memory.
Those cells must come out bit-identical to the exact arithmetic, the rest
within the F64X bound."""
import numpy as np
import pytest

from oracle import core
from tests._helpers import fluid_mask, rel_err
from lbmminiapp_gb300 import Simulation, workloads

pytestmark = pytest.mark.gpu


def perturbed_state(Q, nx, ny, nz, seed):
    rng = np.random.default_rng(seed)
    u = workloads.taylor_green(nx, ny, nz, 0.04, noise=1e-3, seed=seed)
    f = core.equilibrium(Q, np.ones((nz, ny, nx)), u)
    cells = rng.choice(nx * ny * nz, size=12, replace=False)
    fv = f.reshape(Q, -1)
    fv[2, cells[:4]] = 0.3                 # non-rest population above 1/4
    fv[5, cells[4:8]] = -1e-3              # negative population
    fv[:, cells[8:]] = core.equilibrium(Q, np.ones(4), np.array([[0.15] * 4, [0.0] * 4, [0.0] * 4]))
    return f, cells


@pytest.mark.parametrize("Q", [19, 27])
@pytest.mark.parametrize("shape,walls", [((32, 6, 5), False), ((35, 7, 5), True)])
def test_fallback_cells_are_exact(gpu, Q, shape, walls):
    nx, ny, nz = shape
    f0, cells = perturbed_state(Q, nx, ny, nz, seed=Q + nx)
    solid = workloads.channel_mask(nx, ny, nz) if walls else np.zeros((nz, ny, nx), np.uint8)
    per = (1, 0, 1) if walls else (1, 1, 1)
    f0[:, solid.astype(bool)] = 0.0
    out = {}
    for arith in ("f64", "f64x"):
        with Simulation(nx, ny, nz, lattice=Q, pattern="aa", omega=1.0 / 0.6, force=(1e-5, 0, 0), periodic=per,
                        arithmetic=arith) as sim:
            sim.set_solid(solid)
            sim.set_populations(f0, "logical")
            sim.step(1)       # the even step: each cell's own inputs go through the collision
            out[arith] = sim.get_populations("raw")
    m = fluid_mask(solid, Q)
    fluid_cells = [c for c in cells if not solid.ravel()[c]]
    a = out["f64x"].reshape(Q, -1)[:, fluid_cells]
    b = out["f64"].reshape(Q, -1)[:, fluid_cells]
    assert np.array_equal(a, b)
    assert rel_err(out["f64x"], out["f64"], m) < 1e-13


@pytest.mark.parametrize("Q", [19, 27])
def test_fallback_over_several_steps(gpu, Q):
    """Even and odd steps with out-of-range cells: the whole field stays
    within the F64X bound of the exact arithmetic."""
    nx, ny, nz = 32, 6, 5
    f0, _ = perturbed_state(Q, nx, ny, nz, seed=3)
    out = {}
    for arith in ("f64", "f64x"):
        with Simulation(nx, ny, nz, lattice=Q, pattern="aa", omega=1.0 / 0.6, force=(1e-5, 0, 0),
                        arithmetic=arith) as sim:
            sim.set_populations(f0, "logical")
            sim.step(4)
            out[arith] = sim.get_populations("raw")
    assert rel_err(out["f64x"], out["f64"]) < 1e-12
