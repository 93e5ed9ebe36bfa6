"""Pythonic handle over the C ABI: one :class:`Simulation` = one ``lbm_handle``.

Host arrays follow the library's conventions: numpy arrays shaped
``(nz, ny, nx)``; per-direction arrays ``(Q, nz, ny, nx)``; vectors
``(3, nz, ny, nx)``.  Device buffers are owned by the handle (or, for the
kernel-level calls, by the caller).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N

PATTERNS = {"aa": (N.PATTERN_AA, 0), "ab_push": (N.PATTERN_AB, 0), "ab_pull": (N.PATTERN_AB, 1)}


class Simulation:
    def __init__(self, nx, ny, nz, lattice=19, pattern="aa", omega=1.0, force=(0.0, 0.0, 0.0),
                 periodic=(1, 1, 1), storage="f64", arithmetic="auto", unroll=False, device=0,
                 max_device_bytes=0, compact=False):
        if pattern not in PATTERNS:
            raise ValueError(f"pattern must be one of {sorted(PATTERNS)}")
        self.lib = N.lib()
        cfg = N.Config()
        N.check(self.lib.lbm_config_default(ctypes.byref(cfg)))
        cfg.lattice = int(lattice)
        cfg.prop_pattern, cfg.pull = PATTERNS[pattern]
        cfg.unroll = int(bool(unroll))
        cfg.nx, cfg.ny, cfg.nz = int(nx), int(ny), int(nz)
        for d in range(3):
            cfg.periodic[d] = int(bool(periodic[d]))
            cfg.force[d] = float(force[d])
        cfg.omega = float(omega)
        cfg.storage = N.STORAGE_NAMES[storage] if isinstance(storage, str) else int(storage)
        cfg.arithmetic = N.ARITH_NAMES[arithmetic] if isinstance(arithmetic, str) else int(arithmetic)
        cfg.device = int(device)
        cfg.max_device_bytes = int(max_device_bytes)
        cfg.compact = int(bool(compact))
        h = ctypes.c_void_p()
        st = self.lib.lbm_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != N.LBM_OK:
            raise N.LBMError(st, "lbm_create failed (see stderr)")
        self.h = h
        self.cfg = cfg
        self.Q = int(lattice)
        self.pattern = pattern
        self.shape = (int(nz), int(ny), int(nx))
        self.ncell = int(nx) * int(ny) * int(nz)

    # ------------------------------------------------------------ lifetime
    def close(self):
        if getattr(self, "h", None):
            self.lib.lbm_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, st):
        N.check(st, self.h)

    @property
    def info(self) -> N.Info:
        inf = N.Info()
        self._check(self.lib.lbm_get_info(self.h, ctypes.byref(inf)))
        return inf

    @property
    def time_step(self) -> int:
        return int(self.info.time_step)

    @property
    def nfluid(self) -> int:
        return int(self.info.nfluid)

    def set_stream(self, stream_handle: int | None):
        self._check(self.lib.lbm_set_stream(self.h, ctypes.c_void_p(stream_handle or 0)))

    def synchronize(self):
        self._check(self.lib.lbm_synchronize(self.h))

    # ------------------------------------------------------------ geometry
    def set_solid(self, solid):
        if solid is None:
            self._check(self.lib.lbm_set_solid(self.h, None))
            return
        s = np.ascontiguousarray(solid, dtype=np.uint8)
        assert s.shape == self.shape
        self._check(self.lib.lbm_set_solid(self.h, N.ptr(s)))

    def set_force_field(self, field):
        f = None if field is None else np.ascontiguousarray(field, dtype=np.float64)
        if f is not None:
            assert f.shape == (3,) + self.shape
        self._check(self.lib.lbm_set_force_field(self.h, N.ptr(f)))

    def set_porosity(self, porosity):
        p = None if porosity is None else np.ascontiguousarray(porosity, dtype=np.float64)
        if p is not None:
            assert p.shape == self.shape
        self._check(self.lib.lbm_set_porosity(self.h, N.ptr(p)))

    # ------------------------------------------------------------ state
    def init_equilibrium(self, rho=None, u=None):
        r = None if rho is None else np.ascontiguousarray(rho, dtype=np.float64)
        v = None if u is None else np.ascontiguousarray(u, dtype=np.float64)
        self._check(self.lib.lbm_init_equilibrium(self.h, N.ptr(r), N.ptr(v)))

    def set_populations(self, f, layout="logical"):
        a = np.ascontiguousarray(f, dtype=np.float64)
        assert a.shape == (self.Q,) + self.shape
        lay = N.LAYOUT_LOGICAL if layout == "logical" else N.LAYOUT_RAW
        self._check(self.lib.lbm_set_populations(self.h, N.ptr(a), lay))

    def get_populations(self, layout="logical"):
        out = np.empty((self.Q,) + self.shape)
        lay = N.LAYOUT_LOGICAL if layout == "logical" else N.LAYOUT_RAW
        self._check(self.lib.lbm_get_populations(self.h, N.ptr(out), lay))
        return out

    def step(self, n=1):
        self._check(self.lib.lbm_step(self.h, int(n)))

    def macros(self, out=None):
        """(rho, u) with the reference readout semantics; ``out`` may supply
        preallocated (rho, u) float64 arrays (e.g. views of pinned memory)."""
        if out is None:
            rho = np.empty(self.shape)
            u = np.empty((3,) + self.shape)
        else:
            rho, u = out
            assert rho.shape == self.shape and u.shape == (3,) + self.shape
            assert rho.dtype == np.float64 and u.dtype == np.float64
            assert rho.flags.c_contiguous and u.flags.c_contiguous
        self._check(self.lib.lbm_get_macros(self.h, N.ptr(rho), N.ptr(u)))
        return rho, u

    def conserved(self):
        out = np.empty(4)
        self._check(self.lib.lbm_reduce_conserved(self.h, N.ptr(out)))
        return out

    # ------------------------------------------------------------ kernel level
    def population_buffer(self) -> int:
        p = ctypes.c_void_p()
        self._check(self.lib.lbm_population_buffer(self.h, ctypes.byref(p)))
        return int(p.value or 0)

    def timestep_even_force(self, dstrb_ptr: int, start: int, count: int):
        self._check(self.lib.lbm_timestep_even_force(self.h, ctypes.c_void_p(dstrb_ptr), start, count))

    def timestep_odd_force(self, dstrb_ptr: int, start: int, count: int):
        self._check(self.lib.lbm_timestep_odd_force(self.h, ctypes.c_void_p(dstrb_ptr), start, count))

    def timestep_force(self, src_ptr: int, tgt_ptr: int, start: int, count: int):
        self._check(self.lib.lbm_timestep_force(self.h, ctypes.c_void_p(src_ptr), ctypes.c_void_p(tgt_ptr),
                                                start, count))


def cylinder(simulation_size: float):
    """Reference cylinder mask (src/geometries/Geometry.cpp:59-71,112-140) built
    by the library; returns (dims (nx,ny,nz), solid (nz,ny,nx) uint8)."""
    L = N.lib()
    dims = (ctypes.c_int * 3)()
    N.check(L.lbm_geometry_cylinder(float(simulation_size), dims, None))
    nx, ny, nz = dims[0], dims[1], dims[2]
    solid = np.empty((nz, ny, nx), np.uint8)
    N.check(L.lbm_geometry_cylinder(float(simulation_size), dims, N.ptr(solid)))
    return (nx, ny, nz), solid
