"""ctypes wrapper of the reference's own CPU kernels (test oracle).

``oracle/build_ref.sh`` compiles the unmodified lbmminiapp sources plus
``ref_harness.cpp`` into ``oracle/_ref/libref_q{19,27}.so``.  Those libraries
exist only where the reference sources were available at build time;
:func:`available` says whether they can be used here.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
# The reference sources: $LBM_REFERENCE_DIR, else a checkout named "reference"
# beside this repository.
REF_DIR = Path(os.environ.get("LBM_REFERENCE_DIR", str(HERE.parents[1] / "reference")))
OUT = HERE / "_ref"

AA_BASE, AA_UNROLL, AB_PUSH_BASE, AB_PUSH_UNROLL, AB_PULL_BASE, AB_PULL_UNROLL = range(6)

_libs: dict[int, ctypes.CDLL] = {}


def build() -> bool:
    """Build the reference libraries if the sources exist; True when usable."""
    if not (REF_DIR / "src" / "kernels").is_dir():
        return _usable()
    srcs = [HERE / "ref_harness.cpp", HERE / "build_ref.sh", HERE / "ref_overrides.h"]
    newest = max(p.stat().st_mtime for p in srcs)
    if _usable() and all((OUT / f"libref_q{q}.so").stat().st_mtime >= newest for q in (19, 27)):
        return True
    subprocess.run(["bash", str(HERE / "build_ref.sh")], check=True)
    return _usable()


def _usable() -> bool:
    for q in (19, 27):
        p = OUT / f"libref_q{q}.so"
        if not p.exists():
            return False
        try:
            ctypes.CDLL(str(p))
        except OSError:
            return False
    return True


def available() -> bool:
    try:
        return build()
    except (subprocess.CalledProcessError, OSError):
        return False


def lib(Q: int) -> ctypes.CDLL:
    if Q not in _libs:
        L = ctypes.CDLL(str(OUT / f"libref_q{Q}.so"))
        P = ctypes.c_void_p
        L.ref_box_run.argtypes = [ctypes.c_int] * 4 + [P, P, ctypes.c_double, ctypes.c_double, P,
                                                      ctypes.c_int, P, P]
        L.ref_box_run.restype = ctypes.c_int
        L.ref_app_prepare.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double, P, P, P, P]
        L.ref_app_execute.argtypes = [P, P, P, P]
        L.ref_app_execute_compact.argtypes = [P, P, P, P, P]
        _libs[Q] = L
    return _libs[Q]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def box_run(Q, variant, f_init, nsteps, omega, gx, periodic=(1, 1, 1), solid=None):
    """Reference kernels on a dense box; returns (f_raw (Q,nz,ny,nx), seconds)."""
    f_init = np.ascontiguousarray(f_init, dtype=np.float64)
    _, nz, ny, nx = f_init.shape
    per = np.ascontiguousarray(periodic, dtype=np.int32)
    sol = None if solid is None else np.ascontiguousarray(solid, dtype=np.uint8)
    out = np.empty_like(f_init)
    sec = ctypes.c_double(0.0)
    rc = lib(Q).ref_box_run(variant, nx, ny, nz, _ptr(sol), _ptr(per), float(omega), float(gx),
                            _ptr(f_init), int(nsteps), _ptr(out), ctypes.byref(sec))
    if rc:
        raise RuntimeError(f"ref_box_run failed with code {rc}")
    return out, sec.value


def app_run(Q, input_file, omega=1.0, gx=1e-6):
    """The reference's whole single-rank flow on one of its input files.

    Returns dict(dims, nfluid, steps, prop_pattern, rho, u, f_raw, seconds);
    arrays dense (Lz, Ly, Lx) with x the pipe axis."""
    L = lib(Q)
    dims = (ctypes.c_int * 3)()
    nf = ctypes.c_longlong()
    steps = ctypes.c_int()
    pp = ctypes.c_int()
    L.ref_app_prepare(str(input_file).encode(), float(omega), float(gx), dims, ctypes.byref(nf),
                      ctypes.byref(steps), ctypes.byref(pp))
    nx, ny, nz = dims[0], dims[1], dims[2]
    rho = np.empty((nz, ny, nx))
    u = np.empty((3, nz, ny, nx))
    f = np.empty((Q, nz, ny, nx))
    sec = ctypes.c_double()
    L.ref_app_execute(_ptr(rho), _ptr(u), _ptr(f), ctypes.byref(sec))
    return dict(dims=(nx, ny, nz), nfluid=nf.value, steps=steps.value, prop_pattern=pp.value,
                rho=rho, u=u, f_raw=f, seconds=sec.value)


def app_run_compact(Q, input_file, omega=1.0, gx=1e-6):
    """The reference's single-rank flow on one of its input files, returning
    its own compact buffers: dict(dims, nfluid, steps, prop_pattern,
    adjacency [Q, nfluid] int32 (GeometryAAAB::setupAdjacency), fluid_pts
    [nfluid, 3] (i, j, k) in the reference's sorted order, raw_init and
    raw_final [Q, nfluid] (population buffer before and after the run),
    seconds)."""
    L = lib(Q)
    dims = (ctypes.c_int * 3)()
    nf = ctypes.c_longlong()
    steps = ctypes.c_int()
    pp = ctypes.c_int()
    L.ref_app_prepare(str(input_file).encode(), float(omega), float(gx), dims, ctypes.byref(nf),
                      ctypes.byref(steps), ctypes.byref(pp))
    n = nf.value
    adj = np.empty((Q, n), np.int32)
    pts = np.empty((n, 3), np.int32)
    f0 = np.empty((Q, n))
    f1 = np.empty((Q, n))
    sec = ctypes.c_double()
    rc = L.ref_app_execute_compact(_ptr(f0), _ptr(f1), _ptr(adj), _ptr(pts), ctypes.byref(sec))
    if rc:
        raise RuntimeError(f"ref_app_execute_compact failed with code {rc}")
    return dict(dims=(dims[0], dims[1], dims[2]), nfluid=n, steps=steps.value, prop_pattern=pp.value,
                adjacency=adj, fluid_pts=pts, raw_init=f0, raw_final=f1, seconds=sec.value)
