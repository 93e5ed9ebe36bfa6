"""Parity of the CUDA path at the full-size configurations it is credited on.

* C1: 64^3 fully periodic D3Q19 AA, tau 0.8, rho 1, Taylor-Green U 0.05,
  200 steps (reference: src/kernels/KernelAA_SOA_Base.cpp:173-342);
* C2: 256x128x128 D3Q27 channel, AB push and pull, gx 1e-6, tau 0.6, rest
  start, 1000 steps (src/kernels/KernelAB_SOA_Base.cpp:111-186,
  KernelAB_SOA_Pull.cpp:113-194);
* the headline workload (512^3 in the benchmark) at 256^3: D3Q19 AA,
  tau 0.55, Taylor-Green U 0.05 plus uniform 1e-3 noise, 1000 steps.

For C1 and C2 the exact FP64 arithmetic must hash to the reference's digest
(tests/golden/pin_*.npz), so its result is the reference's result, and F64X
must stay within 1e-10 relative (max |a - b| / max |b| over fluid cells) of it
in the raw and logical populations, density and velocity.  The headline workload compares F64X with
the exact FP64 arithmetic on the GPU, which is the reference's result.  The
measured maxima are printed in the pytest summary.
"""
import numpy as np
import pytest

from oracle import core
from lbmminiapp_gb300 import Simulation, workloads
from tests._helpers import fluid_digest, fluid_mask, load_golden, pin_init, rel_err

pytestmark = pytest.mark.gpu

F64X_TOL = 1e-10
PATTERNS = {core.AA: "aa", core.AB_PUSH: "ab_push", core.AB_PULL: "ab_pull"}


def run_gpu(fix, f0, solid, arithmetic):
    nx, ny, nz = (int(v) for v in fix["dims"])
    with Simulation(nx, ny, nz, lattice=int(fix["Q"]), pattern=PATTERNS[int(fix["pattern"])],
                    omega=float(fix["omega"]), force=(float(fix["gx"]), 0.0, 0.0),
                    periodic=tuple(int(v) for v in fix["periodic"]), storage="f64", arithmetic=arithmetic) as sim:
        sim.set_solid(solid)
        sim.set_populations(f0, "logical")
        sim.step(int(fix["steps"]))
        raw = sim.get_populations("raw")
        logical = sim.get_populations("logical")
        rho, u = sim.macros()
    return raw, logical, rho, u


@pytest.mark.parametrize("name", ["pin_c1_q19_aa_tg64", "pin_c2_q27_ab_push_channel", "pin_c2_q27_ab_pull_channel"])
def test_reference_pin(gpu, parity_record, name):
    fix = load_golden(name)
    Q = int(fix["Q"])
    f0, solid = pin_init(fix)
    assert fluid_digest(f0, solid) == str(fix["init_sha256"])
    m, fm = fluid_mask(solid, Q), fluid_mask(solid)
    raw_e, logical_e, rho_e, u_e = run_gpu(fix, f0, solid, "f64")
    # bit-identical: the exact FP64 result is the reference's result
    assert np.array_equal(raw_e.reshape(Q, -1)[:, fix["sample_cells"]], fix["sample_f"])
    assert fluid_digest(raw_e, solid) == str(fix["final_sha256"]), "exact FP64 is not bit-identical"
    raw, logical, rho, u = run_gpu(fix, f0, solid, "f64x")
    errs = {"raw": rel_err(raw, raw_e, m), "logical": rel_err(logical, logical_e, m),
            "rho": rel_err(rho, rho_e, fm), "u": rel_err(u, u_e, np.broadcast_to(fm, u.shape))}
    parity_record(f"{name} F64X vs reference", errs)
    assert max(errs.values()) <= F64X_TOL, errs


def test_c1_readouts_match_oracle_port(gpu):
    """C1 readouts of the exact arithmetic against the oracle port's (which
    hashes to the reference's populations): logical populations bit for bit,
    rho and u to the last bits of the readout sums."""
    fix = load_golden("pin_c1_q19_aa_tg64")
    f0, solid = pin_init(fix)
    steps = int(fix["steps"])
    port, _ = core.run(19, core.AA, f0, steps, float(fix["omega"]), (0, 0, 0), (1, 1, 1), solid)
    assert fluid_digest(port, solid) == str(fix["final_sha256"])
    _, logical, rho, u = run_gpu(fix, f0, solid, "f64")
    assert np.array_equal(logical, core.raw_to_logical(19, core.AA, steps, port, solid, (1, 1, 1)))
    rr, ur = core.readout_macros(19, core.AA, steps, port, solid, (1, 1, 1))
    assert rel_err(rho, rr) < 1e-15 and rel_err(u, ur) < 1e-13


def test_headline_workload_f64x_vs_exact_f64(gpu, parity_record):
    n, steps = 256, 1000
    u0 = workloads.taylor_green(n, n, n, U=0.05, noise=1e-3, seed=2024)
    out = {}
    for arith in ("f64", "f64x"):
        with Simulation(n, n, n, lattice=19, pattern="aa", omega=1.0 / 0.55, force=(0, 0, 0),
                        arithmetic=arith) as sim:
            sim.init_equilibrium(None, u0)
            sim.step(steps)
            out[arith] = (sim.get_populations("raw"), *sim.macros())
    (f_e, rho_e, u_e), (f_x, rho_x, u_x) = out["f64"], out["f64x"]
    errs = {"raw": rel_err(f_x, f_e), "rho": rel_err(rho_x, rho_e), "u": rel_err(u_x, u_e)}
    parity_record("D3Q19 AA 256^3 tau 0.55 TG+noise 1000 steps, F64X vs exact FP64", errs)
    assert max(errs.values()) <= F64X_TOL, errs
