"""The oracle (C restatement) against the reference's own kernels and the
golden fixtures; CPU only."""
import numpy as np
import pytest

from oracle import core, ref
from tests._helpers import fluid_mask, golden_cases, load_golden, rel_err
from lbmminiapp_gb300 import workloads


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_golden(name):
    g = load_golden(name)
    Q, pattern = int(g["Q"]), int(g["pattern"])
    out, _ = core.run(Q, pattern, g["f_init"], int(g["steps"]), float(g["omega"]), (float(g["gx"]), 0, 0),
                      tuple(g["periodic"]), g["solid"], bool(g["compat"]))
    m = fluid_mask(g["solid"], Q)
    assert np.array_equal(np.isnan(out), np.isnan(g["f_raw"]))
    err = rel_err(out, g["f_raw"], m)
    if int(g["variant"]) in (ref.AA_BASE, ref.AB_PUSH_BASE, ref.AB_PULL_BASE):
        # same operation order, no FMA contraction: bit-identical
        assert np.array_equal(out[m], g["f_raw"][m]), err
    else:
        # Unroll kernels associate omega*w*rho differently: last-bit differences
        assert err < 1e-14


needs_ref = pytest.mark.skipif(not ref.available(), reason="reference sources not present")


@needs_ref
@pytest.mark.parametrize("Q,variant,pattern,compat", [
    (19, ref.AA_BASE, core.AA, 0), (19, ref.AA_UNROLL, core.AA, 1), (19, ref.AB_PUSH_BASE, core.AB_PUSH, 0),
    (19, ref.AB_PULL_UNROLL, core.AB_PULL, 0), (27, ref.AA_BASE, core.AA, 0), (27, ref.AB_PULL_BASE, core.AB_PULL, 0),
])
def test_oracle_vs_reference_random(Q, variant, pattern, compat):
    rng = np.random.default_rng(Q * 10 + variant)
    nx, ny, nz = 7, 6, 5
    solid = (rng.random((nz, ny, nx)) < 0.15).astype(np.uint8)
    u = workloads.taylor_green(nx, ny, nz, 0.04, noise=2e-3, seed=variant)
    f0 = core.equilibrium(Q, 1.0 + 0.01 * rng.random((nz, ny, nx)), u)
    per = (1, 0, 1)
    r, _ = ref.box_run(Q, variant, f0, 6, 1.0 / 0.65, 3e-6, per, solid)
    o, _ = core.run(Q, pattern, f0, 6, 1.0 / 0.65, (3e-6, 0, 0), per, solid, bool(compat))
    m = fluid_mask(solid, Q)
    if variant in (ref.AA_BASE, ref.AB_PUSH_BASE, ref.AB_PULL_BASE):
        assert np.array_equal(o[m], r[m])
    else:
        assert rel_err(o, r, m) < 1e-14


@needs_ref
def test_reference_cylinder_app_matches_library_geometry(tmp_path):
    """The reference's whole flow on its own input file, 20 steps: the cylinder
    mask and the readout match the library geometry builder and the oracle."""
    import lbmminiapp_gb300 as lbm
    src = ref.REF_DIR / "test" / "2_input_aa_unroll.txt"
    inp = tmp_path / "in.txt"
    inp.write_text(src.read_text().replace("timesteps 1000", "timesteps 20"))
    out = ref.app_run(19, inp, omega=1.0, gx=1e-6)
    dims, solid = lbm.cylinder(2.0)
    assert dims == out["dims"]
    assert int((solid == 0).sum()) == out["nfluid"] == 153216
    assert np.array_equal(np.isnan(out["rho"]), solid.astype(bool))
    # oracle on the same geometry (x-periodic only, AA, compat weights)
    c, opp, w = core.stencil(19)
    f0 = np.broadcast_to(w[:, None, None, None], (19,) + solid.shape).copy()
    o, _ = core.run(19, core.AA, f0, 20, 1.0, (1e-6, 0, 0), (1, 0, 0), solid, True)
    m = fluid_mask(solid, 19)
    assert rel_err(o, out["f_raw"], m) < 1e-14
