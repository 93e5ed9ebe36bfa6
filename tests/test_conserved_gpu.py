"""lbm_reduce_conserved: mass and momentum sums over fluid cells.

Cells whose populations all lie in [2^-32, 1) are summed exactly as 128-bit
fixed-point integers (units of 2^-84) and rounded once, so the totals are the
exact sums of the logical populations to within one rounding; other cells go
to FP64 accumulators.  Checked against exact rational sums made here from the
logical populations the library returns."""
import math
from fractions import Fraction

import numpy as np
import pytest

from oracle import core
from lbmminiapp_gb300 import Simulation, workloads

pytestmark = pytest.mark.gpu


def exact_sums(Q, f, fluid):
    """Exact sums of f and c_d f over the fluid cells, as Fractions."""
    c, _, _ = core.stencil(Q)
    vals = f[:, fluid]                       # [Q, nfluid]
    scaled = [[int(v) for v in np.ldexp(vals[s], 84)] for s in range(Q)]
    per_dir = [sum(row) for row in scaled]
    mass = Fraction(sum(per_dir), 1 << 84)
    mom = [Fraction(sum(int(c[s, d]) * per_dir[s] for s in range(Q)), 1 << 84) for d in range(3)]
    return [mass] + mom


@pytest.mark.parametrize("Q,pattern,storage,steps", [
    (19, "aa", "f64", 3),
    (19, "aa", "f64", 4),
    (27, "ab_pull", "f64", 2),
    (27, "aa", "f32", 5),
    (19, "ab_push", "f16", 3),
])
def test_sums_are_exact_for_physical_states(gpu, Q, pattern, storage, steps):
    nx, ny, nz = 30, 20, 14
    solid = workloads.channel_mask(nx, ny, nz)
    u = workloads.taylor_green(nx, ny, nz, 0.05, noise=1e-3, seed=Q + steps)
    u[:, solid.astype(bool)] = 0
    with Simulation(nx, ny, nz, lattice=Q, pattern=pattern, omega=1.5, force=(1e-5, 2e-6, 0),
                    periodic=(1, 0, 1), storage=storage) as sim:
        sim.set_solid(solid)
        sim.init_equilibrium(None, u)
        sim.step(steps)
        got = sim.conserved()
        f = sim.get_populations("logical")
    fluid = solid == 0
    assert np.all((f[:, fluid] >= 2.0 ** -32) & (f[:, fluid] < 1.0))
    for k, ex in enumerate(exact_sums(Q, f, fluid)):
        want = float(ex)
        # one rounding of the 128-bit total, plus one of its low word
        assert abs(got[k] - want) <= 2 * math.ulp(max(abs(want), 1e-300)), (k, got[k], want)


def test_cells_outside_the_fixed_point_range_are_summed_in_fp64(gpu):
    """Negative and zero populations (not a physical state, but a caller may
    set one) take the FP64 accumulators; the totals still agree with the
    exact sums to FP64 accuracy."""
    nx, ny, nz = 16, 12, 10
    Q = 19
    f = core.equilibrium(Q, np.ones((nz, ny, nx)), workloads.taylor_green(nx, ny, nz, 0.05))
    f[3, 2, 5, 7] = -0.01
    f[7, 9, 1, 2] = 0.0
    f[0, 4, 4, 4] = 1.5
    with Simulation(nx, ny, nz, lattice=Q, pattern="ab_push") as sim:
        sim.set_populations(f)
        got = sim.conserved()
        back = sim.get_populations("logical")
    fluid = np.ones((nz, ny, nx), bool)
    c, _, _ = core.stencil(Q)
    want = [back[:, fluid].sum()] + [(back[:, fluid] * c[:, d, None]).sum() for d in range(3)]
    assert abs(got[0] - want[0]) <= 1e-13 * abs(want[0])
    assert np.all(np.abs(got[1:] - np.array(want[1:])) <= 1e-13 * abs(want[0]))
