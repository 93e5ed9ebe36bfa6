import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a library)")


@pytest.fixture(scope="session")
def gpu():
    """The CUDA library, loaded (and built in-tree if needed).  GPU tests fail
    loudly when it cannot be built or loaded: there is no CPU fallback."""
    import lbmminiapp_gb300 as lbm
    lbm.lib()
    return lbm


_PARITY = []


@pytest.fixture
def parity_record():
    """record(name, {quantity: max relative error}): printed in the summary."""
    def record(name, errs):
        _PARITY.append((name, dict(errs)))
    return record


def pytest_terminal_summary(terminalreporter):
    if not _PARITY:
        return
    terminalreporter.section("parity maxima (max |a - b| / max |b|)")
    for name, errs in _PARITY:
        terminalreporter.write_line(f"{name}: " + ", ".join(f"{k} {v:.2e}" for k, v in errs.items()))
