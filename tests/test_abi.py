"""The C-ABI library loads and exports every entry point the header declares
(no GPU needed: nothing here launches a kernel)."""
import ctypes
import re
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(lbm_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_declared_symbols():
    from lbmminiapp_gb300 import _native
    lib = _native.lib()
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    # every header declaration has a ctypes prototype in the binding
    assert set(names) <= set(_native.exported_symbols())


def test_status_strings_and_defaults():
    from lbmminiapp_gb300 import _native as N
    lib = N.lib()
    assert lib.lbm_status_string(0) == b"ok"
    assert b"diverged" in lib.lbm_status_string(4)
    cfg = N.Config()
    assert lib.lbm_config_default(ctypes.byref(cfg)) == 0
    assert cfg.lattice == 19 and cfg.prop_pattern == N.PATTERN_AA and cfg.omega == 1.0
    assert cfg.force[0] == 0.000001   # the reference's _GRAVITY_
    assert lib.lbm_config_default(None) == 1


def test_create_rejects_bad_config_without_gpu_work():
    """Argument validation happens before any device call."""
    from lbmminiapp_gb300 import _native as N
    lib = N.lib()
    cfg = N.Config()
    lib.lbm_config_default(ctypes.byref(cfg))
    h = ctypes.c_void_p()
    for field, value in [("lattice", 15), ("omega", 2.5), ("prop_pattern", 3), ("storage", 9), ("nx", 0)]:
        c2 = N.Config.from_buffer_copy(cfg)
        setattr(c2, field, value)
        st = lib.lbm_create(ctypes.byref(c2), ctypes.byref(h))
        assert st == 1, (field, st)
        assert not h.value


def test_cylinder_geometry_host_only():
    import lbmminiapp_gb300 as lbm
    dims, solid = lbm.cylinder(2.0)
    assert dims == (168, 35, 35)
    assert int((solid == 0).sum()) == 153216
    dims4, solid4 = lbm.cylinder(4.0)
    assert int((solid4 == 0).sum()) == 1154496
    # mask is constant along the pipe axis x and symmetric in y, z
    assert np.array_equal(solid[:, :, 0:1].repeat(168, axis=2), solid)
    assert np.array_equal(solid, solid.transpose(1, 0, 2))
