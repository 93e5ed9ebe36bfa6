"""Failure detection through the C ABI (no GPU fault is provoked: every
failure is made on the host or in the data, and must come back as a status
code with a message while the context stays usable)."""
import numpy as np
import pytest

from oracle import core
from lbmminiapp_gb300 import LBMError, Simulation, workloads

pytestmark = pytest.mark.gpu


def test_device_memory_cap_gives_out_of_memory(gpu):
    # 64^3 D3Q19 FP64 needs about 40 MB for its population buffer alone
    with pytest.raises(LBMError) as e:
        Simulation(64, 64, 64, max_device_bytes=1 << 20)
    assert e.value.status == 2
    with Simulation(64, 64, 64, max_device_bytes=1 << 30) as sim:   # the same shape under a roomy cap
        sim.init_equilibrium()
        sim.step(2)
        assert sim.conserved()[0] == pytest.approx(64 ** 3, rel=1e-13)


@pytest.mark.parametrize("storage", ["f64", "f16"])
def test_non_finite_state_is_reported_as_diverged(gpu, storage):
    nx, ny, nz = 16, 8, 6
    f = core.equilibrium(19, np.ones((nz, ny, nx)), workloads.taylor_green(nx, ny, nz, 0.05))
    f[4, 3, 2, 5] = np.nan
    with Simulation(nx, ny, nz, storage=storage) as sim:
        sim.set_populations(f)
        sim.step(3)
        with pytest.raises(LBMError) as e:
            sim.conserved()
        assert e.value.status == 4 and "conserved sum" in str(e.value)
        # the handle (and the context) stay usable
        sim.init_equilibrium()
        sim.step(2)
        assert np.isfinite(sim.conserved()).all()


def test_bad_calls_give_status_codes(gpu):
    with Simulation(12, 8, 6, pattern="aa") as sim:
        buf = sim.population_buffer()
        with pytest.raises(LBMError) as e:
            sim.timestep_even_force(buf, 0, sim.ncell + 1)
        assert e.value.status == 1
        with pytest.raises(LBMError) as e:
            sim.timestep_force(buf, buf + 8, 0, 10)      # AB call on an AA handle
        assert e.value.status == 6
        with pytest.raises(LBMError) as e:
            sim.set_porosity(np.full((6, 8, 12), 1.5))
        assert e.value.status == 1
    with pytest.raises(LBMError) as e:
        Simulation(12, 8, 6, storage="f16", arithmetic="f64")
    assert e.value.status == 5
