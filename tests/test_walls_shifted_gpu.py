"""Shifted FP32 / BF16 / FP16 storage with walls and solids.

The full-grid step runs the pipelined one-cell-per-lane kernel (rows of 32
cells, full and ragged: nx = 14 and 13); kernel-level range calls run the
one-cell-per-thread kernel.  Both are checked against the FP64 oracle (the
tolerance is the storage format's rounding, relative to max |f| over fluid
cells, after 5 steps) and against each other."""
import numpy as np
import pytest

from oracle import core
from tests._helpers import fluid_mask, rel_err
from lbmminiapp_gb300 import Simulation, workloads

pytestmark = pytest.mark.gpu

PIDS = {"aa": core.AA, "ab_push": core.AB_PUSH, "ab_pull": core.AB_PULL}
TOL = {"f32": 1e-6, "bf16": 2e-3, "f16": 2e-4}


def case(Q, nx, seed=4):
    rng = np.random.default_rng(seed)
    ny, nz = 9, 7
    solid = workloads.channel_mask(nx, ny, nz) | (rng.random((nz, ny, nx)) < 0.12).astype(np.uint8)
    u = workloads.taylor_green(nx, ny, nz, 0.04, noise=2e-3, seed=seed)
    u[:, solid.astype(bool)] = 0
    f0 = core.equilibrium(Q, 1.0 + 0.01 * rng.random((nz, ny, nx)), u)
    return (nx, ny, nz), solid, f0


@pytest.mark.parametrize("Q", [19, 27])
@pytest.mark.parametrize("pattern", ["aa", "ab_push", "ab_pull"])
@pytest.mark.parametrize("storage", ["f32", "bf16", "f16"])
@pytest.mark.parametrize("nx", [14, 13])
def test_walls_and_solids_match_oracle(gpu, Q, pattern, storage, nx):
    dims, solid, f0 = case(Q, nx)
    per, omega, F, steps = (1, 0, 1), 1.0 / 0.7, (1e-5, 0, 0), 5
    ref, _ = core.run(Q, PIDS[pattern], f0, steps, omega, F, per, solid)
    ref_log = core.raw_to_logical(Q, PIDS[pattern], steps, ref, solid, per)
    with Simulation(*dims, lattice=Q, pattern=pattern, omega=omega, force=F, periodic=per, storage=storage) as sim:
        sim.set_solid(solid)
        sim.set_populations(f0, "logical")
        sim.step(steps)
        out = sim.get_populations("logical")
    m = fluid_mask(solid, Q)
    assert rel_err(out, ref_log, m) < TOL[storage]
    assert np.isnan(out[:, solid.astype(bool)]).all()


@pytest.mark.parametrize("storage", ["f32", "bf16", "f16"])
@pytest.mark.parametrize("nx", [14, 13])
def test_full_grid_kernels_match_per_cell_kernel(gpu, storage, nx):
    """Full-grid AA steps against the same steps as kernel-level range calls
    (one cell per thread): the same FP32 collision on the same stored values."""
    dims, solid, f0 = case(19, nx, seed=9)
    kw = dict(lattice=19, pattern="aa", omega=1.4, force=(2e-6, 0, 0), periodic=(1, 0, 1), storage=storage)
    with Simulation(*dims, **kw) as a, Simulation(*dims, **kw) as b:
        for s in (a, b):
            s.set_solid(solid)
            s.set_populations(f0, "logical")
        a.step(4)
        buf = b.population_buffer()
        n = b.ncell
        for t in range(4):
            call = b.timestep_even_force if t % 2 == 0 else b.timestep_odd_force
            call(buf, 0, 301)
            call(buf, 301, n - 301)
        b.synchronize()
        ra = a.get_populations("logical")
        rb = b.get_populations("logical")
    m = fluid_mask(solid, 19)
    assert rel_err(ra, rb, m) < 1e-6
