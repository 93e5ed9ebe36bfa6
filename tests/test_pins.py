"""Full-size parity pins (CPU part): the C1 and C2 fixtures made from the
reference itself, and the oracle port against the C1 pin.

Each pin fixture (tests/golden/make_golden.py --pins) keeps the SHA-256 of the
reference's final populations over the fluid cells and a sample of 1024 cells;
the GPU tests (tests/test_pins_gpu.py) compare the CUDA path with the same
digests and with the oracle port run there.
"""
import numpy as np
import pytest

from oracle import core
from tests._helpers import fluid_digest, load_golden, pin_init

PINS = ["pin_c1_q19_aa_tg64", "pin_c2_q27_ab_push_channel", "pin_c2_q27_ab_pull_channel"]


@pytest.mark.parametrize("name", PINS)
def test_pin_initial_state_rebuilds_exactly(name):
    """The initial state rebuilt from the fixture's tables is the one the
    reference ran from, bit for bit."""
    fix = load_golden(name)
    f0, solid = pin_init(fix)
    assert fluid_digest(f0, solid) == str(fix["init_sha256"])
    assert fix["sample_f"].shape == (int(fix["Q"]), 1024)
    assert not solid.ravel()[fix["sample_cells"]].any()


def test_c1_oracle_port_is_the_reference():
    """64^3 periodic D3Q19 AA, tau 0.8, Taylor-Green U 0.05, 200 steps: the
    oracle port's final populations hash to the reference Base kernels'
    (src/kernels/KernelAA_SOA_Base.cpp:173-342)."""
    fix = load_golden("pin_c1_q19_aa_tg64")
    f0, solid = pin_init(fix)
    out, _ = core.run(19, core.AA, f0, int(fix["steps"]), float(fix["omega"]), (0.0, 0.0, 0.0), (1, 1, 1), solid)
    assert np.array_equal(out.reshape(19, -1)[:, fix["sample_cells"]], fix["sample_f"])
    assert fluid_digest(out, solid) == str(fix["final_sha256"])
