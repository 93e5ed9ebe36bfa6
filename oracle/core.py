"""ctypes wrapper of oracle/lbm_oracle.c and numpy helpers (test oracle).

Array conventions shared with the product library and the tests:

* dense cell index ``c = x + nx*(y + ny*z)``; numpy arrays are shaped
  ``(nz, ny, nx)`` and per-direction arrays ``(Q, nz, ny, nx)``;
* "raw" arrays hold the slot contents of the population buffer exactly as the
  reference stores them (AA: direction s in slot opp(s) at even time;
  AB pull: post-collision values not yet streamed);
* "logical" arrays hold direction s of each cell, post-stream and
  pre-collision.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liblbm_oracle.so"

AA, AB_PUSH, AB_PULL = 0, 1, 2

# Velocity sets in the reference's order (src/lattices/LatticeD3Q19.cpp:5-88,
# src/lattices/LatticeD3Q27.cpp:5-120).
C19 = np.array([
    [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
    [1, 1, 0], [1, -1, 0], [1, 0, 1], [1, 0, -1], [-1, 1, 0], [-1, -1, 0],
    [-1, 0, 1], [-1, 0, -1], [0, 1, 1], [0, 1, -1], [0, -1, 1], [0, -1, -1],
    [0, 0, 0]], dtype=np.int64)
C27 = np.array([
    [1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1],
    [1, 1, 0], [1, -1, 0], [1, 0, 1], [1, 0, -1], [-1, 1, 0], [-1, -1, 0],
    [-1, 0, 1], [-1, 0, -1], [0, 1, 1], [0, 1, -1], [0, -1, 1], [0, -1, -1],
    [1, 1, 1], [1, 1, -1], [1, -1, 1], [1, -1, -1], [-1, 1, 1], [-1, 1, -1],
    [-1, -1, 1], [-1, -1, -1], [0, 0, 0]], dtype=np.int64)


def stencil(Q: int):
    """(c[Q,3], opp[Q], w[Q]) for Q in (19, 27)."""
    c = C19 if Q == 19 else C27 if Q == 27 else None
    if c is None:
        raise ValueError("Q must be 19 or 27")
    opp = np.array([int(np.flatnonzero((c == -c[s]).all(axis=1))[0]) for s in range(Q)])
    n2 = (c * c).sum(axis=1)
    if Q == 19:
        table = {0: 1.0 / 3.0, 1: 1.0 / 18.0, 2: 1.0 / 36.0}
    else:
        table = {0: 8.0 / 27.0, 1: 2.0 / 27.0, 2: 1.0 / 54.0, 3: 1.0 / 216.0}
    w = np.array([table[int(k)] for k in n2])
    return c, opp, w


def build(force: bool = False) -> Path:
    """Compile lbm_oracle.c into oracle/liblbm_oracle.so (gcc, OpenMP, no FMA
    contraction so x86-64 and aarch64 give identical bits)."""
    src = HERE / "lbm_oracle.c"
    if LIB_PATH.exists() and not force and LIB_PATH.stat().st_mtime >= src.stat().st_mtime:
        return LIB_PATH
    tmp = LIB_PATH.with_suffix(f".so.tmp{os.getpid()}")
    cmd = [os.environ.get("CC", "gcc"), "-O2", "-std=gnu11", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", str(src), "-o", str(tmp), "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        P = ctypes.c_void_p
        L.lbm_oracle_run.argtypes = [ctypes.c_int] * 3 + [ctypes.c_int] * 3 + [P, P, ctypes.c_double,
                                                                              P, P, P, P, ctypes.c_int,
                                                                              ctypes.c_int, P, P]
        L.lbm_oracle_run.restype = ctypes.c_int
        L.lbm_oracle_max_threads.restype = ctypes.c_int
        L.lbm_oracle_create.argtypes = [ctypes.c_int] * 6 + [P, P, ctypes.c_double, P, P, P, P, ctypes.c_int]
        L.lbm_oracle_create.restype = ctypes.c_void_p
        L.lbm_oracle_step.argtypes = [P, ctypes.c_int, P]
        L.lbm_oracle_read.argtypes = [P, P]
        L.lbm_oracle_destroy.argtypes = [P]
        L.lbm_oracle_fluid_count.argtypes = [P]
        L.lbm_oracle_fluid_count.restype = ctypes.c_longlong
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def run(Q, pattern, f_init, nsteps, omega, force=(0.0, 0.0, 0.0), periodic=(1, 1, 1),
        solid=None, compat_rest_weight=False, force_field=None, porosity=None, nthreads=0):
    """Run the C restatement; returns (f_raw (Q,nz,ny,nx), loop seconds)."""
    f_init = np.ascontiguousarray(f_init, dtype=np.float64)
    _, nz, ny, nx = f_init.shape
    assert f_init.shape[0] == Q
    per = np.ascontiguousarray(periodic, dtype=np.int32)
    sol = None if solid is None else np.ascontiguousarray(solid, dtype=np.uint8)
    frc = np.ascontiguousarray(force, dtype=np.float64)
    ff = None if force_field is None else np.ascontiguousarray(force_field, dtype=np.float64)
    por = None if porosity is None else np.ascontiguousarray(porosity, dtype=np.float64)
    out = np.empty_like(f_init)
    sec = ctypes.c_double(0.0)
    rc = lib().lbm_oracle_run(Q, pattern, int(bool(compat_rest_weight)), nx, ny, nz, _ptr(per),
                              _ptr(sol), float(omega), _ptr(frc), _ptr(ff), _ptr(por),
                              _ptr(f_init), int(nsteps), int(nthreads), _ptr(out),
                              ctypes.byref(sec))
    if rc:
        raise RuntimeError(f"lbm_oracle_run failed with code {rc}")
    return out, sec.value


class Runner:
    """Persistent oracle state for timing individual steps (CPU baseline)."""

    def __init__(self, Q, pattern, f_init, omega, force=(0.0, 0.0, 0.0), periodic=(1, 1, 1), solid=None,
                 compat_rest_weight=False, nthreads=0):
        self._keep = [np.ascontiguousarray(periodic, dtype=np.int32),
                      None if solid is None else np.ascontiguousarray(solid, dtype=np.uint8),
                      np.ascontiguousarray(force, dtype=np.float64),
                      np.ascontiguousarray(f_init, dtype=np.float64)]
        per, sol, frc, f0 = self._keep
        _, nz, ny, nx = f0.shape
        self.Q = Q
        self.shape = (nz, ny, nx)
        self.h = lib().lbm_oracle_create(Q, pattern, int(bool(compat_rest_weight)), nx, ny, nz, _ptr(per),
                                         _ptr(sol), float(omega), _ptr(frc), None, None, _ptr(f0),
                                         int(nthreads))
        if not self.h:
            raise RuntimeError("lbm_oracle_create failed")
        self._keep[3] = None  # initial populations were copied

    @property
    def nfluid(self) -> int:
        return int(lib().lbm_oracle_fluid_count(self.h))

    def step(self, n=1) -> float:
        sec = ctypes.c_double(0.0)
        if lib().lbm_oracle_step(self.h, int(n), ctypes.byref(sec)):
            raise RuntimeError("lbm_oracle_step failed")
        return sec.value

    def read(self):
        out = np.empty((self.Q,) + self.shape)
        lib().lbm_oracle_read(self.h, _ptr(out))
        return out

    def close(self):
        if self.h:
            lib().lbm_oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()


def max_threads() -> int:
    return int(lib().lbm_oracle_max_threads())


def equilibrium(Q, rho, u):
    """Reference equilibrium w rho (1 + cu + cu^2/2 - uu/2), cu = 3 c.u, uu = 3 u.u
    (src/kernels/KernelAA_SOA_Base.cpp:210-236); u has shape (3, ...)."""
    c, _, w = stencil(Q)
    rho = np.asarray(rho, dtype=np.float64)
    u = np.asarray(u, dtype=np.float64)
    uu = 3.0 * (u[0] * u[0] + u[1] * u[1] + u[2] * u[2])
    out = np.empty((Q,) + rho.shape)
    for s in range(Q):
        cu = 3.0 * (c[s, 0] * u[0] + c[s, 1] * u[1] + c[s, 2] * u[2])
        out[s] = w[s] * rho * (1.0 + cu + 0.5 * cu * cu - 0.5 * uu)
    return out


def pull_gather(Q, raw, solid=None, periodic=(1, 1, 1)):
    """Direction s of cell x = slot s at x - c_s, or the own cell's slot opp(s)
    when x - c_s is solid or outside a non-periodic face (the adjacency rule of
    src/geometries/GeometryAAAB.cpp:50-84)."""
    c, opp, _ = stencil(Q)
    _, nz, ny, nx = raw.shape
    out = np.empty_like(raw)
    zz, yy, xx = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    sol = np.zeros((nz, ny, nx), bool) if solid is None else np.asarray(solid, bool)
    dims = (nx, ny, nz)
    for s in range(Q):
        src = [xx - c[s, 0], yy - c[s, 1], zz - c[s, 2]]
        inside = np.ones_like(xx, dtype=bool)
        for d in range(3):
            if periodic[d]:
                src[d] = src[d] % dims[d]
            inside &= (src[d] >= 0) & (src[d] < dims[d])
        sx, sy, sz = (np.clip(src[0], 0, nx - 1), np.clip(src[1], 0, ny - 1),
                      np.clip(src[2], 0, nz - 1))
        blocked = ~inside | sol[sz, sy, sx]
        out[s] = np.where(blocked, raw[opp[s]], raw[s][sz, sy, sx])
    out[:, sol] = np.nan
    return out


def raw_to_logical(Q, pattern, step, raw, solid=None, periodic=(1, 1, 1)):
    """Post-stream, pre-collision populations from the raw buffer.

    AA, even step: direction s sits in slot opp(s) of its own cell
    (src/propagation/PropagationAA.cpp:224-240); AA odd step and AB pull:
    streamed through the pull gather (:241-257); AB push: slot s as stored
    (src/propagation/PropagationAB.cpp:227-241)."""
    _, opp, _ = stencil(Q)
    if pattern == AB_PUSH:
        return raw.copy()
    if pattern == AA and step % 2 == 0:
        return raw[opp].copy()
    return pull_gather(Q, raw, solid, periodic)


def readout_macros(Q, pattern, step, raw, solid=None, periodic=(1, 1, 1)):
    """rho and u = sum(c f)/rho (no F/2 shift) with the reference readout
    semantics (PropagationAA.cpp:218-327, PropagationAB.cpp:222-281): AA reads
    the streamed populations, AB (push and pull) the stored buffer."""
    c, _, _ = stencil(Q)
    f = raw_to_logical(Q, pattern, step, raw, solid, periodic) if pattern == AA else raw
    rho = np.zeros(f.shape[1:])
    m = np.zeros((3,) + f.shape[1:])
    for s in range(Q):
        rho += f[s]
        for d in range(3):
            m[d] += f[s] * c[s, d]
    return rho, m / rho
