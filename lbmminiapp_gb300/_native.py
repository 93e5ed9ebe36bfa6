"""ctypes binding of ``liblbm_gb300.so`` (the C ABI in ``include/lbm_gb300.h``).

The library is the only compute path: when it cannot be loaded every call
raises; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "liblbm_gb300.so"

LBM_OK = 0
(LBM_ERR_INVALID_ARGUMENT, LBM_ERR_OUT_OF_MEMORY, LBM_ERR_CUDA, LBM_ERR_DIVERGED, LBM_ERR_UNSUPPORTED,
 LBM_ERR_STATE) = range(1, 7)
STATUS_NAMES = {
    0: "LBM_OK", 1: "LBM_ERR_INVALID_ARGUMENT", 2: "LBM_ERR_OUT_OF_MEMORY", 3: "LBM_ERR_CUDA",
    4: "LBM_ERR_DIVERGED", 5: "LBM_ERR_UNSUPPORTED", 6: "LBM_ERR_STATE",
}

PATTERN_AB, PATTERN_AA = 0, 1
STORE_F64, STORE_F32, STORE_BF16, STORE_F16 = 0, 1, 2, 3
ARITH_AUTO, ARITH_F64, ARITH_F64X, ARITH_F32 = 0, 1, 2, 3
LAYOUT_RAW, LAYOUT_LOGICAL = 0, 1
LOSS_NONE, LOSS_VELOCITY, LOSS_ENERGY = 0, 1, 2

STORAGE_NAMES = {"f64": STORE_F64, "f32": STORE_F32, "bf16": STORE_BF16, "f16": STORE_F16}
ARITH_NAMES = {"auto": ARITH_AUTO, "f64": ARITH_F64, "f64x": ARITH_F64X, "f32": ARITH_F32}


class Config(ctypes.Structure):
    _fields_ = [
        ("lattice", ctypes.c_int), ("prop_pattern", ctypes.c_int), ("pull", ctypes.c_int),
        ("unroll", ctypes.c_int), ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("periodic", ctypes.c_int * 3), ("omega", ctypes.c_double), ("force", ctypes.c_double * 3),
        ("storage", ctypes.c_int), ("arithmetic", ctypes.c_int), ("device", ctypes.c_int),
        ("compact", ctypes.c_int), ("max_device_bytes", ctypes.c_uint64),
    ]


class Info(ctypes.Structure):
    _fields_ = [
        ("ncell", ctypes.c_int64), ("nfluid", ctypes.c_int64), ("time_step", ctypes.c_int64),
        ("plane_stride", ctypes.c_int64), ("buffer_bytes", ctypes.c_uint64),
        ("device_bytes", ctypes.c_uint64), ("bytes_per_update", ctypes.c_int),
        ("lattice", ctypes.c_int), ("storage", ctypes.c_int), ("arithmetic", ctypes.c_int),
    ]


# name -> (restype, argtypes)
_P = ctypes.c_void_p
_I64 = ctypes.c_int64
_SIGNATURES = {
    "lbm_config_default": (ctypes.c_int, [ctypes.POINTER(Config)]),
    "lbm_create": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.POINTER(_P)]),
    "lbm_destroy": (None, [_P]),
    "lbm_last_error": (ctypes.c_char_p, [_P]),
    "lbm_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "lbm_get_info": (ctypes.c_int, [_P, ctypes.POINTER(Info)]),
    "lbm_set_stream": (ctypes.c_int, [_P, _P]),
    "lbm_synchronize": (ctypes.c_int, [_P]),
    "lbm_set_solid": (ctypes.c_int, [_P, _P]),
    "lbm_geometry_cylinder": (ctypes.c_int, [ctypes.c_double, ctypes.POINTER(ctypes.c_int), _P]),
    "lbm_set_force_field": (ctypes.c_int, [_P, _P]),
    "lbm_set_porosity": (ctypes.c_int, [_P, _P]),
    "lbm_init_equilibrium": (ctypes.c_int, [_P, _P, _P]),
    "lbm_set_populations": (ctypes.c_int, [_P, _P, ctypes.c_int]),
    "lbm_get_populations": (ctypes.c_int, [_P, _P, ctypes.c_int]),
    "lbm_step": (ctypes.c_int, [_P, ctypes.c_int]),
    "lbm_get_macros": (ctypes.c_int, [_P, _P, _P]),
    "lbm_reduce_conserved": (ctypes.c_int, [_P, _P]),
    "lbm_timestep_even_force": (ctypes.c_int, [_P, _P, _I64, _I64]),
    "lbm_timestep_odd_force": (ctypes.c_int, [_P, _P, _I64, _I64]),
    "lbm_timestep_force": (ctypes.c_int, [_P, _P, _P, _I64, _I64]),
    "lbm_population_buffer": (ctypes.c_int, [_P, ctypes.POINTER(_P)]),
    "lbm_copy_state": (ctypes.c_int, [_P, _P, ctypes.c_int]),
    "lbm_set_fields_device": (ctypes.c_int, [_P, _P, _P]),
    "lbm_loss": (ctypes.c_int, [_P, _P, ctypes.c_int, _P, ctypes.c_double, _P]),
    "lbm_adjoint_step": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int, ctypes.c_int, _P, ctypes.c_double, _P, _P]),
    "lbm_adjoint_step_f32": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int, ctypes.c_int, _P, ctypes.c_double, _P, _P]),
    "lbm_sparse_create": (ctypes.c_int, [ctypes.POINTER(Config), _I64, _P, ctypes.POINTER(_P)]),
    "lbm_sparse_destroy": (None, [_P]),
    "lbm_sparse_last_error": (ctypes.c_char_p, [_P]),
    "lbm_sparse_set_stream": (ctypes.c_int, [_P, _P]),
    "lbm_sparse_timestep_even_force": (ctypes.c_int, [_P, _P, _I64, _I64]),
    "lbm_sparse_timestep_odd_force": (ctypes.c_int, [_P, _P, _I64, _I64]),
    "lbm_sparse_timestep_force": (ctypes.c_int, [_P, _P, _P, _I64, _I64]),
    "lbm_reduce_conserved_noalloc": (ctypes.c_int, [ctypes.c_int] * 5 + [_I64, _P, _P, _P, ctypes.c_int, _P, _P]),
}

_lib = None


class LBMError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def library_path() -> Path:
    return Path(os.environ.get("LBM_GB300_LIB", str(LIB_PATH)))


def lib(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load liblbm_gb300.so (building it in-tree when missing)."""
    global _lib
    if _lib is None:
        path = library_path()
        if not path.exists() and build_if_missing:
            from . import build as _build
            _build.build()
        if not path.exists():
            raise RuntimeError(f"CUDA library {path} is missing; run lbmminiapp_gb300/build.py")
        L = ctypes.CDLL(str(path))
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return sorted(_SIGNATURES)


def ptr(a):
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data_as(ctypes.c_void_p)
    return ctypes.c_void_p(int(a))


def check(status: int, handle=None):
    if status != LBM_OK:
        msg = lib().lbm_last_error(handle).decode() if handle is not None else ""
        raise LBMError(status, msg or lib().lbm_status_string(status).decode())
