"""Mixed-precision storage error against FP64 storage (Taylor-Green + noise,
D3Q19 AA, tau = 0.55) on a 64^3 box over 200 steps.  Bounds: FP32 5e-5 (the
same order as a plain float32 emulation of the scheme, ~1.5e-5 on 32^3),
FP16 (shifted, scaled by 2^15) 1e-3 and BF16 5e-2 relative L2 velocity error;
total mass within 1e-6 relative (FP16, BF16) and 1e-9 (FP32)."""
import pytest

pytestmark = pytest.mark.gpu


def test_error_table_small(gpu):
    from lbmminiapp_gb300.accuracy import error_table
    t = error_table(n=64, steps=200)
    assert abs(t["f64"]["mass_drift_rel"]) < 1e-12
    assert t["f32"]["u_rel_l2"] < 5e-5 and abs(t["f32"]["mass_rel"]) < 1e-7
    assert t["f16"]["u_rel_l2"] < 1e-3 and abs(t["f16"]["mass_rel"]) < 1e-6
    assert t["bf16"]["u_rel_l2"] < 5e-2 and abs(t["bf16"]["mass_rel"]) < 1e-4
