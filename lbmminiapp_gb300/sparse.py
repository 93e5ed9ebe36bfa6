"""Compact fluid-only layout: the reference's own buffers and adjacency list.

The reference keeps populations only for fluid points (direction ``s`` of
fluid point ``i`` at ``dstrb[nFluid*s + i]``) and streams through the int32
adjacency list of ``GeometryAAAB::setupAdjacency``
(src/geometries/GeometryAAAB.cpp:18-124).  :class:`SparseKernels` wraps an
``lbm_sparse_handle`` (``include/lbm_gb300.h``): the reference's kernel steps
on caller-owned device buffers in that layout.  :func:`build_adjacency`
builds the list from a solid mask with the same semantics, in any fluid
order, for callers that do not have the reference's geometry.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native as N
from .simulation import PATTERNS

_C19 = np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1], [1, 1, 0], [1, -1, 0],
                 [1, 0, 1], [1, 0, -1], [-1, 1, 0], [-1, -1, 0], [-1, 0, 1], [-1, 0, -1], [0, 1, 1], [0, 1, -1],
                 [0, -1, 1], [0, -1, -1], [0, 0, 0]])
_C27 = np.concatenate([_C19[:18], np.array([[1, 1, 1], [1, 1, -1], [1, -1, 1], [1, -1, -1], [-1, 1, 1],
                                            [-1, 1, -1], [-1, -1, 1], [-1, -1, -1], [0, 0, 0]])])


def velocities(Q: int) -> np.ndarray:
    """Velocity set in the reference's order (src/lattices/LatticeD3Q19.cpp,
    LatticeD3Q27.cpp)."""
    if Q == 19:
        return _C19
    if Q == 27:
        return _C27
    raise ValueError("Q must be 19 or 27")


def opposite(Q: int) -> np.ndarray:
    c = velocities(Q)
    return np.array([int(np.flatnonzero((c == -c[s]).all(axis=1))[0]) for s in range(Q)])


def build_adjacency(solid, periodic=(1, 1, 1), pattern="aa", lattice=19, order=None):
    """Fluid list and adjacency with the semantics of
    GeometryAAAB::setupAdjacency (src/geometries/GeometryAAAB.cpp:44-84).

    solid: (nz, ny, nx) mask, nonzero = solid.  The neighbour of direction s
    is x + c_s for AB push and x - c_s for AA and AB pull; a periodic axis
    wraps; a solid or out-of-box neighbour maps to the own slot opp(s).
    order: optional permutation of the fluid cells (default: x fastest).

    Returns (fluid_cells, adjacency): the dense cell index x + nx*(y + ny*z)
    of each fluid point, and an int32 array [Q, nfluid] of element indices
    nfluid*s' + j.
    """
    solid = np.asarray(solid).astype(bool)
    nz, ny, nx = solid.shape
    Q = int(lattice)
    c = velocities(Q)
    opp = opposite(Q)
    fluid = np.flatnonzero(~solid.ravel())
    if order is not None:
        fluid = fluid[np.asarray(order)]
    n = fluid.size
    if Q * n >= 2 ** 31:
        raise ValueError("Q * nfluid must stay below 2^31 (int32 element indices)")
    index = np.full(solid.size, -1, np.int64)
    index[fluid] = np.arange(n)
    x = fluid % nx
    y = (fluid // nx) % ny
    z = fluid // (nx * ny)
    push = PATTERNS[pattern] == (N.PATTERN_AB, 0)
    adj = np.empty((Q, n), np.int32)
    for s in range(Q):
        d = c[s] if push else c[opp[s]]
        coords = []
        inside = np.ones(n, bool)
        for k, (v, L) in enumerate(zip((x, y, z), (nx, ny, nz))):
            w = v + d[k]
            if periodic[k]:
                w = np.mod(w, L)
            else:
                inside &= (w >= 0) & (w < L)
                w = np.clip(w, 0, L - 1)
            coords.append(w)
        nb = index[coords[0] + nx * (coords[1] + ny * coords[2])]
        nb = np.where(inside, nb, -1)
        own = n * opp[s] + np.arange(n)
        adj[s] = np.where(nb >= 0, n * s + nb, own)
    return fluid, adj


class SparseKernels:
    """One ``lbm_sparse_handle``: the reference's kernel steps on compact
    device buffers.  Buffer arguments are device pointers (ints) or objects
    with ``data_ptr()`` (e.g. torch CUDA tensors) holding Q*nfluid doubles."""

    def __init__(self, adjacency, lattice=19, pattern="aa", omega=1.0, force=(0.0, 0.0, 0.0), arithmetic="auto",
                 unroll=False, device=0):
        adjacency = np.ascontiguousarray(adjacency, dtype=np.int32)
        if adjacency.ndim != 2 or adjacency.shape[0] != int(lattice):
            raise ValueError("adjacency must be [Q, nfluid]")
        self.lib = N.lib()
        cfg = N.Config()
        N.check(self.lib.lbm_config_default(ctypes.byref(cfg)))
        cfg.lattice = int(lattice)
        cfg.prop_pattern, cfg.pull = PATTERNS[pattern]
        cfg.unroll = int(bool(unroll))
        cfg.omega = float(omega)
        for d in range(3):
            cfg.force[d] = float(force[d])
        cfg.storage = N.STORE_F64
        cfg.arithmetic = N.ARITH_NAMES[arithmetic] if isinstance(arithmetic, str) else int(arithmetic)
        cfg.device = int(device)
        h = ctypes.c_void_p()
        st = self.lib.lbm_sparse_create(ctypes.byref(cfg), int(adjacency.shape[1]), N.ptr(adjacency),
                                        ctypes.byref(h))
        if st != N.LBM_OK:
            raise N.LBMError(st, "lbm_sparse_create failed")
        self.h = h
        self.Q = int(lattice)
        self.pattern = pattern
        self.nfluid = int(adjacency.shape[1])

    def close(self):
        if getattr(self, "h", None):
            self.lib.lbm_sparse_destroy(self.h)
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
        if st != N.LBM_OK:
            raise N.LBMError(st, self.lib.lbm_sparse_last_error(self.h).decode())

    @staticmethod
    def _dev(buf):
        return ctypes.c_void_p(int(buf.data_ptr()) if hasattr(buf, "data_ptr") else int(buf))

    def set_stream(self, stream):
        s = stream if isinstance(stream, int) else getattr(stream, "cuda_stream", 0)
        self._check(self.lib.lbm_sparse_set_stream(self.h, ctypes.c_void_p(int(s))))

    def timestep_even_force(self, dstrb, start=0, count=None):
        count = self.nfluid - start if count is None else count
        self._check(self.lib.lbm_sparse_timestep_even_force(self.h, self._dev(dstrb), int(start), int(count)))

    def timestep_odd_force(self, dstrb, start=0, count=None):
        count = self.nfluid - start if count is None else count
        self._check(self.lib.lbm_sparse_timestep_odd_force(self.h, self._dev(dstrb), int(start), int(count)))

    def timestep_force(self, src, tgt, start=0, count=None):
        count = self.nfluid - start if count is None else count
        self._check(self.lib.lbm_sparse_timestep_force(self.h, self._dev(src), self._dev(tgt), int(start),
                                                       int(count)))

    def run(self, buffers, nsteps, t0=0):
        """nsteps whole-range steps in the reference's time-loop order
        (PropagationAA.cpp:169-183, PropagationAB.cpp:182-188).  buffers: one
        buffer for AA, [src, tgt] for AB (swapped after every step, as the
        reference swaps its pointers).  Returns the buffer holding the latest
        state."""
        if self.pattern == "aa":
            buf = buffers[0] if isinstance(buffers, (list, tuple)) else buffers
            for t in range(t0, t0 + nsteps):
                (self.timestep_even_force if t % 2 == 0 else self.timestep_odd_force)(buf)
            return buf
        src, tgt = buffers
        for _ in range(nsteps):
            self.timestep_force(src, tgt)
            src, tgt = tgt, src
        return src
