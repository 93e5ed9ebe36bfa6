"""Degenerate and ragged box shapes through every full-grid kernel (pipelined
FP64/F64X, shifted-storage pair and pipelined kernels) against the oracle:
extents of 1 and 2 (a periodic neighbour is the cell itself or its only
other cell), rows shorter than and not a multiple of the 32-cell tile."""
import numpy as np
import pytest

from oracle import core
from tests._helpers import fluid_mask, rel_err
from lbmminiapp_gb300 import Simulation, workloads

pytestmark = pytest.mark.gpu

SHAPES = [(1, 5, 4), (6, 1, 3), (5, 4, 1), (2, 2, 2), (1, 1, 1), (33, 3, 2), (64, 2, 3)]
PIDS = {"aa": core.AA, "ab_push": core.AB_PUSH, "ab_pull": core.AB_PULL}


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("pattern", ["aa", "ab_pull"])
@pytest.mark.parametrize("arithmetic,storage,tol", [("f64x", "f64", 1e-12), ("auto", "f32", 1e-6)])
def test_small_and_ragged_boxes(gpu, shape, pattern, arithmetic, storage, tol):
    nx, ny, nz = shape
    rng = np.random.default_rng(nx * 100 + ny * 10 + nz)
    u = 0.03 * rng.uniform(-1, 1, (3, nz, ny, nx))
    f0 = core.equilibrium(19, 1.0 + 0.01 * rng.random((nz, ny, nx)), u)
    steps, omega, F = 5, 1.0 / 0.7, (1e-5, 0, 0)
    ref, _ = core.run(19, PIDS[pattern], f0, steps, omega, F, (1, 1, 1))
    ref_log = core.raw_to_logical(19, PIDS[pattern], steps, ref, None, (1, 1, 1))
    with Simulation(nx, ny, nz, lattice=19, pattern=pattern, omega=omega, force=F, storage=storage,
                    arithmetic=arithmetic) as sim:
        sim.set_populations(f0)
        sim.step(steps)
        out = sim.get_populations("logical")
    assert rel_err(out, ref_log) < tol


@pytest.mark.parametrize("shape", [(1, 6, 5), (33, 5, 4)])
def test_small_boxes_with_walls(gpu, shape):
    nx, ny, nz = shape
    solid = workloads.channel_mask(nx, ny, nz)
    rng = np.random.default_rng(3)
    u = 0.03 * rng.uniform(-1, 1, (3, nz, ny, nx))
    u[:, solid.astype(bool)] = 0
    f0 = core.equilibrium(27, np.ones((nz, ny, nx)), u)
    ref, _ = core.run(27, core.AA, f0, 4, 1.0 / 0.6, (1e-5, 0, 0), (1, 0, 1), solid)
    ref_log = core.raw_to_logical(27, core.AA, 4, ref, solid, (1, 0, 1))
    with Simulation(nx, ny, nz, lattice=27, pattern="aa", omega=1.0 / 0.6, force=(1e-5, 0, 0),
                    periodic=(1, 0, 1)) as sim:
        sim.set_solid(solid)
        sim.set_populations(f0)
        sim.step(4)
        out = sim.get_populations("logical")
    assert rel_err(out, ref_log, fluid_mask(solid, 27)) < 1e-12
