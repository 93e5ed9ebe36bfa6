"""Sphere-packing permeability and mean-flux porosity gradient (no reference
counterpart): reduced-precision forward/adjoint against the FP64 ones.

The full-size study (384^3 D3Q27, 2000 steps) runs as ``bench.py --porous``;
these tests run the same pipeline on a 48^3 packing of spheres of radius 3-6.
"""
import numpy as np
import pytest

from lbmminiapp_gb300 import porous, workloads
from lbmminiapp_gb300.simulation import Simulation

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("storage", ["f64", "f16"])
def test_aa_and_ab_push_hold_the_same_populations(gpu, storage):
    """The adjoint differentiates the AB-push rollout; the AA run it stands for
    must hold the same populations after every step."""
    solid, _, _ = workloads.sphere_packing(32, 0.3, 3.0, 5.0, seed=11)
    out = []
    for pattern in ("aa", "ab_push"):
        with Simulation(32, 32, 32, lattice=27, pattern=pattern, omega=1 / 0.7, force=(1e-5, 0, 0),
                        storage=storage, arithmetic="f64" if storage == "f64" else "auto") as sim:
            sim.set_solid(solid)
            sim.init_equilibrium()
            sim.step(41)
            out.append(sim.get_populations())
    assert np.array_equal(out[0], out[1], equal_nan=True)


def test_porous_scaled_study(gpu):
    solid, _, _ = workloads.sphere_packing(48, 0.35, 3.0, 6.0, seed=3)
    tau, gx, steps = 0.7, 1e-5, 300
    f64 = porous.forward(solid, tau, gx, steps, storage="f64", arithmetic="f64")
    f16 = porous.forward(solid, tau, gx, steps, storage="f16")
    k_err = abs(f16["permeability"] - f64["permeability"]) / f64["permeability"]
    L64, g64, _ = porous.flux_gradient(solid, tau, gx, steps, (100, 10), storage="f64", adjoint="f64",
                                       arithmetic="f64")
    L16, g16, _ = porous.flux_gradient(solid, tau, gx, steps, (100, 10), storage="f16", adjoint="f32")
    fluid = ~solid.astype(bool)
    e = porous.gradient_errors(g16, g64, fluid)
    print(f"k64 {f64['permeability']:.6e} k16 {f16['permeability']:.6e} rel err {k_err:.2e} "
          f"grad {e}")
    # the AB-push rollout's loss is the AA run's mean flux
    assert abs(L64 - f64["mean_ux"]) <= 1e-12 * abs(L64)
    assert f64["permeability"] > 0
    # measured on GB300: k 1.4e-4, gradient rel L2 1.3e-4
    assert k_err < 1e-3
    assert e["rel_l2"] < 1e-3 and e["corr"] > 0.9999
    # dL/ds < 0 wherever flow passes: blocking a cell lowers the mean flux
    assert (g64[fluid] <= 1e-12 * np.abs(g64).max()).mean() > 0.95
