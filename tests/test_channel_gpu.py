"""D3Q27 AB push and pull in the 256 x 128 x 128 channel (solid rows y = 0 and
y = 127, half-way walls at y = 0.5 and 126.5, periodic x and z), g_x = 1e-6,
tau = 0.6, fluid at rest.

* 100 steps against the oracle (C restatement of the reference kernels) on the
  full grid: populations within 1e-10 relative (F64X arithmetic);
* 1000 steps against the start-up plane Poiseuille series
      u(eta, t) = g/(2 nu) eta (H - eta)
                  - sum_{n odd} 4 g H^2/(nu pi^3 n^3) sin(n pi eta/H) exp(-nu n^2 pi^2 t/H^2)
  with eta = y - 0.5, H = 126, nu = (tau - 1/2)/3: the x/z-averaged physical
  velocity (with the F/2 shift) within 0.5 % of the series maximum.
"""
import numpy as np
import pytest

from oracle import core
from lbmminiapp_gb300 import Simulation, workloads
from tests._helpers import fluid_mask, rel_err

pytestmark = pytest.mark.gpu

NX, NY, NZ = 256, 128, 128
TAU = 0.6
G = 1e-6


def channel_sim(pattern):
    sim = Simulation(NX, NY, NZ, lattice=27, pattern=pattern, omega=1.0 / TAU, force=(G, 0, 0), periodic=(1, 0, 1))
    sim.set_solid(workloads.channel_mask(NX, NY, NZ))
    sim.init_equilibrium()
    return sim


@pytest.mark.parametrize("pattern", ["ab_push", "ab_pull"])
def test_channel_matches_oracle_full_grid(gpu, pattern):
    solid = workloads.channel_mask(NX, NY, NZ)
    _, _, w = core.stencil(27)
    f0 = np.broadcast_to(w[:, None, None, None], (27, NZ, NY, NX)).copy()
    pid = core.AB_PUSH if pattern == "ab_push" else core.AB_PULL
    ref, _ = core.run(27, pid, f0, 100, 1.0 / TAU, (G, 0, 0), (1, 0, 1), solid)
    with channel_sim(pattern) as sim:
        sim.step(100)
        raw = sim.get_populations("raw")
    assert rel_err(raw, ref, fluid_mask(solid, 27)) < 1e-10


def startup_poiseuille(eta, t, H, nu, g, nmax=4001):
    u = g / (2 * nu) * eta * (H - eta)
    for n in range(1, nmax, 2):
        u -= 4 * g * H * H / (nu * np.pi ** 3 * n ** 3) * np.sin(n * np.pi * eta / H) * np.exp(
            -nu * n * n * np.pi * np.pi * t / (H * H))
    return u


@pytest.mark.parametrize("pattern", ["ab_push", "ab_pull"])
def test_channel_startup_poiseuille(gpu, pattern):
    steps = 1000
    with channel_sim(pattern) as sim:
        sim.step(steps)
        rho, u = sim.macros()
    fl = slice(1, NY - 1)
    ux = np.nanmean(u[0][:, fl, :], axis=(0, 2)) + G / 2 / np.nanmean(rho[:, fl, :], axis=(0, 2))
    eta = np.arange(1, NY - 1) - 0.5
    nu = (TAU - 0.5) / 3
    ref = startup_poiseuille(eta, steps, NY - 2, nu, G)
    assert ref.max() == pytest.approx(G * steps, rel=1e-3)   # bulk still accelerating freely
    assert np.abs(ux - ref).max() < 5e-3 * ref.max()
