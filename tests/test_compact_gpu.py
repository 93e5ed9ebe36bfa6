"""Compact fluid-only storage (Simulation(..., compact=True)): AA steps with
shifted FP32 / BF16 / FP16 storage on populations of the fluid cells only.

* Against the dense layout with the same storage: the same FP32 collision on
  the same inputs, so raw and logical populations, macros and the FP64
  conservation sums are bit-identical (walls, random solids, ragged rows,
  rows of one and two cells, odd and even step counts, a geometry change
  mid-run), and at full size on the 384^3 sphere packing (D3Q27 FP16).
* Against the FP64 oracle on a sphere packing: the storage format's error.
"""
import ctypes

import numpy as np
import pytest

from oracle import core
from lbmminiapp_gb300 import Simulation, workloads
from lbmminiapp_gb300 import _native as N
from tests._helpers import fluid_mask, rel_err

pytestmark = pytest.mark.gpu


def case(Q, dims, walls, solid_frac, seed):
    nx, ny, nz = dims
    rng = np.random.default_rng(seed)
    solid = workloads.channel_mask(nx, ny, nz) if walls else np.zeros((nz, ny, nx), np.uint8)
    solid |= (rng.random((nz, ny, nx)) < solid_frac).astype(np.uint8)
    u = workloads.taylor_green(nx, ny, nz, 0.04, noise=2e-3, seed=seed)
    u[:, solid.astype(bool)] = 0
    f0 = core.equilibrium(Q, 1.0 + 0.01 * rng.random((nz, ny, nx)), u)
    return solid, f0


def run(dims, Q, storage, solid, f0, steps, per, compact, force=(1e-5, 0, 0)):
    with Simulation(*dims, lattice=Q, pattern="aa", omega=1.0 / 0.7, force=force, periodic=per, storage=storage,
                    compact=compact) as sim:
        sim.set_solid(solid)
        sim.set_populations(f0, "logical")
        sim.step(steps)
        out = {"raw": sim.get_populations("raw"), "logical": sim.get_populations("logical")}
        out["rho"], out["u"] = sim.macros()
        out["cons"] = sim.conserved()
        out["nfluid"] = sim.nfluid
    return out


GEOMETRIES = {
    "channel_ragged": ((13, 9, 7), (1, 0, 1), True, 0.12),
    "periodic_porous": ((40, 10, 6), (1, 1, 1), False, 0.35),
    "rows_of_one": ((1, 8, 6), (1, 1, 1), False, 0.2),
    "rows_of_two": ((2, 7, 5), (1, 0, 1), True, 0.1),
    "open_x": ((20, 6, 5), (0, 1, 1), False, 0.15),
}


@pytest.mark.parametrize("Q", [19, 27])
@pytest.mark.parametrize("storage", ["f16", "f32", "bf16"])
@pytest.mark.parametrize("geometry", sorted(GEOMETRIES))
@pytest.mark.parametrize("steps", [1, 2, 7])
def test_compact_equals_dense(gpu, Q, storage, geometry, steps):
    dims, per, walls, frac = GEOMETRIES[geometry]
    solid, f0 = case(Q, dims, walls, frac, seed=Q + steps)
    a = run(dims, Q, storage, solid, f0, steps, per, compact=False)
    b = run(dims, Q, storage, solid, f0, steps, per, compact=True)
    assert a["nfluid"] == b["nfluid"] == int((solid == 0).sum())
    for k in ("raw", "logical", "rho", "u", "cons"):
        assert np.array_equal(a[k], b[k], equal_nan=True), k


@pytest.mark.parametrize("Q", [19, 27])
def test_compact_long_sparse_rows_equal_dense(gpu, Q):
    """Rows whose fluid cells lie 9 to 13 apart: 32 of them span more than 255
    cells in x, so the row tiles split at the 255-cell span (their per-lane
    counts are bytes); denser rows and a solid row around them; x open and
    periodic."""
    nx, ny, nz = 700, 4, 3
    rng = np.random.default_rng(11)
    solid = np.zeros((nz, ny, nx), np.uint8)
    for z in range(nz):
        for y in range(ny):
            if (y + z) % 2 == 0:
                row = np.ones(nx, np.uint8)
                x = int(rng.integers(0, 9))
                while x < nx:
                    row[x] = 0
                    x += int(rng.integers(9, 14))
                solid[z, y] = row
            else:
                solid[z, y] = (rng.random(nx) < 0.3).astype(np.uint8)
    solid[1, 2, :] = 1
    u = workloads.taylor_green(nx, ny, nz, 0.04, noise=2e-3, seed=4)
    u[:, solid.astype(bool)] = 0
    f0 = core.equilibrium(Q, 1.0 + 0.01 * rng.random((nz, ny, nx)), u)
    for per in ((1, 1, 1), (0, 1, 1)):
        a = run((nx, ny, nz), Q, "f16", solid, f0, 5, per, compact=False)
        b = run((nx, ny, nz), Q, "f16", solid, f0, 5, per, compact=True)
        for k in ("raw", "logical", "rho", "u", "cons"):
            assert np.array_equal(a[k], b[k], equal_nan=True), (per, k)


def test_compact_without_force_equals_dense(gpu):
    dims, per = (24, 8, 6), (1, 1, 1)
    solid, f0 = case(27, dims, False, 0.3, seed=3)
    a = run(dims, 27, "f16", solid, f0, 6, per, compact=False, force=(0, 0, 0))
    b = run(dims, 27, "f16", solid, f0, 6, per, compact=True, force=(0, 0, 0))
    assert np.array_equal(a["raw"], b["raw"], equal_nan=True)


def test_geometry_change_mid_run(gpu):
    """The state carries over a new solid mask the same way in both layouts."""
    dims, per = (17, 9, 6), (1, 0, 1)
    solid, f0 = case(19, dims, True, 0.1, seed=9)
    solid2 = solid.copy()
    solid2[:, 4, 3:9] = 1
    outs = []
    for compact in (False, True):
        with Simulation(*dims, lattice=19, pattern="aa", omega=1.3, force=(1e-5, 0, 0), periodic=per,
                        storage="f16", compact=compact) as sim:
            sim.set_solid(solid)
            sim.set_populations(f0, "logical")
            sim.step(3)
            sim.set_solid(solid2)
            sim.step(4)
            outs.append(sim.get_populations("raw"))
    assert np.array_equal(outs[0], outs[1], equal_nan=True)


def test_compact_spheres_close_to_fp64_oracle(gpu):
    """D3Q27 AA on a periodic sphere packing (48^3, radius 4-6, solid fraction
    0.35), gx 1e-6, tau 0.7, 40 steps from a Taylor-Green state: FP16 and FP32
    compact storage against the FP64 oracle (velocity relative to max |u|)."""
    n = 48
    solid, _, _ = workloads.sphere_packing(n, 0.35, 4.0, 6.0, seed=5)
    u = workloads.taylor_green(n, n, n, 0.03)
    u[:, solid.astype(bool)] = 0
    f0 = core.equilibrium(27, np.ones((n, n, n)), u)
    ref, _ = core.run(27, core.AA, f0, 40, 1.0 / 0.7, (1e-6, 0, 0), (1, 1, 1), solid)
    rr, ur = core.readout_macros(27, core.AA, 40, ref, solid, (1, 1, 1))
    fm = fluid_mask(solid)
    for storage, tol in (("f16", 2e-3), ("f32", 1e-5)):
        with Simulation(n, n, n, lattice=27, pattern="aa", omega=1.0 / 0.7, force=(1e-6, 0, 0), storage=storage,
                        compact=True) as sim:
            sim.set_solid(solid)
            sim.set_populations(f0, "logical")
            sim.step(40)
            rho, uu = sim.macros()
        assert rel_err(uu, ur, np.broadcast_to(fm, uu.shape)) < tol, storage
        assert np.nanmax(np.abs(rho - rr)) < 10 * tol


def test_compact_full_size_sphere_packing(gpu):
    """The 384^3 D3Q27 FP16 sphere packing (solid fraction 0.35, radius 6-12):
    compact and dense states are bit-identical after an odd and an even
    number of steps (compared on the device)."""
    import torch
    n = 384
    solid, _, _ = workloads.sphere_packing(n, 0.35, 6.0, 12.0, seed=2024)
    sims = []
    for compact in (False, True):
        sim = Simulation(n, n, n, lattice=27, pattern="aa", omega=1.0 / 0.7, force=(1e-6, 0, 0), storage="f16",
                         compact=compact)
        sim.set_solid(solid)
        sim.init_equilibrium()
        sims.append(sim)
    try:
        for steps in (3, 1):
            states = []
            for sim in sims:
                sim.step(steps)
                t = torch.empty(int(sim.info.buffer_bytes), dtype=torch.uint8, device="cuda")
                sim.synchronize()
                torch.cuda.synchronize()
                N.check(sim.lib.lbm_copy_state(sim.h, ctypes.c_void_p(t.data_ptr()), 0), sim.h)
                sim.synchronize()
                states.append(t)
            assert torch.equal(states[0], states[1]), steps
            del states
    finally:
        for sim in sims:
            sim.close()


def test_compact_rules(gpu):
    def status(**kw):
        try:
            Simulation(8, 8, 8, compact=True, **kw).close()
            return N.LBM_OK
        except N.LBMError as e:
            return e.status
    assert status(pattern="ab_push", storage="f16") == N.LBM_ERR_UNSUPPORTED
    assert status(pattern="aa", storage="f64") == N.LBM_ERR_UNSUPPORTED
    assert status(pattern="aa", storage="f16") == N.LBM_OK
    with Simulation(8, 8, 8, storage="f32", compact=True) as sim:
        with pytest.raises(N.LBMError):
            sim.set_porosity(np.zeros((8, 8, 8)))
        with pytest.raises(N.LBMError):
            sim.set_force_field(np.zeros((3, 8, 8, 8)))
        with pytest.raises(N.LBMError):
            sim.population_buffer()
