"""Checkpoint and restart: a state read out after t steps and loaded into a
fresh handle continues bit for bit like the uninterrupted run (FP64 storage).  AA saves the
logical populations (a fresh handle starts at even parity; the logical layout
is parity-free); AB saves the raw buffer (for AB pull it holds post-collision
values, which the logical readout would stream once more)."""
import numpy as np
import pytest

from oracle import core
from lbmminiapp_gb300 import Simulation, workloads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("pattern", ["aa", "ab_push", "ab_pull"])
@pytest.mark.parametrize("arithmetic,storage", [("f64", "f64"), ("f64x", "f64"), ("auto", "f32")])
@pytest.mark.parametrize("t_save", [4, 5])
def test_restart_from_logical_state(gpu, pattern, arithmetic, storage, t_save):
    nx, ny, nz = 32, 9, 6
    solid = workloads.channel_mask(nx, ny, nz)
    u = workloads.taylor_green(nx, ny, nz, 0.04, noise=1e-3, seed=2)
    u[:, solid.astype(bool)] = 0
    f0 = core.equilibrium(19, np.ones((nz, ny, nx)), u)
    kw = dict(lattice=19, pattern=pattern, omega=1.0 / 0.7, force=(1e-5, 0, 0), periodic=(1, 0, 1),
              arithmetic=arithmetic, storage=storage)
    with Simulation(nx, ny, nz, **kw) as whole:
        whole.set_solid(solid)
        whole.set_populations(f0)
        whole.step(9)
        ref = whole.get_populations("logical")
    with Simulation(nx, ny, nz, **kw) as first:
        first.set_solid(solid)
        first.set_populations(f0)
        first.step(t_save)
        layout = "logical" if pattern == "aa" else "raw"
        saved = first.get_populations(layout)
    with Simulation(nx, ny, nz, **kw) as second:
        second.set_solid(solid)
        second.set_populations(saved, layout)
        second.step(9 - t_save)
        out = second.get_populations("logical")
    fluid = ~solid.astype(bool)
    if storage == "f64":
        assert np.array_equal(out[:, fluid], ref[:, fluid])
    else:
        # the host readout adds w back in double; a stored FP32 value g returns
        # exactly unless |g| is far below w's rounding error
        assert np.abs(out[:, fluid] - ref[:, fluid]).max() < 1e-9
