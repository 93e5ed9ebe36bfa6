"""The reference-side shims (integration/*.hh) compile against the unmodified
reference headers, link with the reference's own sources and the library, and
run the reference's set-up flow on its own input files.  CPU test: skipped where
the reference sources are absent; without a GPU the shims stop at lbm_create and
report the library's status through their exception."""
import ctypes
import subprocess
from pathlib import Path

import pytest

from oracle import ref

ROOT = Path(__file__).resolve().parents[1]
needs_ref = pytest.mark.skipif(not (ref.REF_DIR / "src" / "kernels").is_dir(), reason="reference sources not present")


@pytest.fixture(scope="module")
def shims():
    from lbmminiapp_gb300 import build
    build.build()
    subprocess.run(["bash", str(ROOT / "integration" / "build_shims.sh")], check=True)
    libs = {}
    for Q in (19, 27):
        L = ctypes.CDLL(str(ROOT / "oracle" / "_ref" / f"libgb300_shims_q{Q}.so"))
        L.gb300_shim_check.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
        L.gb300_shim_check.restype = ctypes.c_int
        libs[Q] = L
    return libs


def gpu_present():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@needs_ref
@pytest.mark.parametrize("Q", [19, 27])
@pytest.mark.parametrize("input_name", ["2_input_aa_unroll.txt", "2_input_ab_unroll.txt", "2_input_ab_pull_unroll.txt"])
def test_shims_run_the_reference_flow(shims, Q, input_name):
    msg = ctypes.create_string_buffer(1024)
    stage = shims[Q].gb300_shim_check(str(ref.REF_DIR / "test" / input_name).encode(), msg, len(msg))
    if gpu_present():
        assert stage == 3, msg.value
    else:
        assert stage == 0
        assert msg.value.decode().startswith("lbm_create: "), msg.value
