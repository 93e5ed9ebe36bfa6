"""Shared test helpers: golden fixture loading and error metrics."""
from __future__ import annotations

import hashlib
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
PATTERN_NAMES = {0: "aa", 1: "ab_push", 2: "ab_pull"}


def golden_cases():
    """Box / channel cases (reference kernels on a harness geometry)."""
    return sorted(p.stem for p in GOLDEN.glob("*.npz") if not p.stem.startswith(("cylinder_", "sparse_", "pin_")))


def cylinder_cases():
    """The reference's whole app flow on its cylinder (centre plane kept)."""
    return sorted(p.stem for p in GOLDEN.glob("cylinder_*.npz"))


def sparse_cases():
    """The reference's own compact buffers and adjacency (cylinder, size 0.25)."""
    return sorted(p.stem for p in GOLDEN.glob("sparse_*.npz"))


def load_golden(name):
    z = np.load(GOLDEN / f"{name}.npz")
    return {k: z[k] for k in z.files}


def rel_err(a, b, mask=None):
    """max |a - b| / max |b| over cells where mask (or b) is finite."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    m = np.isfinite(b) if mask is None else mask
    m = np.broadcast_to(m, b.shape)
    denom = np.abs(b[m]).max()
    return float(np.abs(a[m] - b[m]).max() / denom) if denom > 0 else float(np.abs(a[m] - b[m]).max())


def fluid_mask(solid, Q=None):
    m = ~np.asarray(solid, bool)
    return m if Q is None else np.broadcast_to(m, (Q,) + m.shape)


def tg_tables(nx, ny, nz):
    """1-D factors of the Taylor-Green vortex (workloads.taylor_green) as stored
    in the pin fixtures."""
    kx, ky, kz = 2 * np.pi / nx, 2 * np.pi / ny, 2 * np.pi / nz
    x, y, z = np.arange(nx), np.arange(ny), np.arange(nz)
    return dict(sin_x=np.sin(kx * x), cos_x=np.cos(kx * x), sin_y=np.sin(ky * y), cos_y=np.cos(ky * y),
                cos_z=np.cos(kz * z))


def pin_init(fix):
    """(f_init (Q, nz, ny, nx), solid) of a pin fixture: equilibrium at rho = 1
    of the Taylor-Green field built from the stored tables (the operation order
    of workloads.taylor_green), or the rest state; solid rows y = 0 and
    y = ny - 1 when the fixture has walls."""
    from oracle import core
    from lbmminiapp_gb300 import workloads
    Q = int(fix["Q"])
    nx, ny, nz = (int(v) for v in fix["dims"])
    U = float(fix["U"])
    u = np.zeros((3, nz, ny, nx))
    if U:
        cz, cy, sy, sx, cx = fix["cos_z"], fix["cos_y"], fix["sin_y"], fix["sin_x"], fix["cos_x"]
        u[0] = U * (cz[:, None, None] * cy[None, :, None]) * sx[None, None, :]
        u[1] = -U * (cz[:, None, None] * sy[None, :, None]) * cx[None, None, :]
    solid = workloads.channel_mask(nx, ny, nz) if int(fix["walls"]) else np.zeros((nz, ny, nx), np.uint8)
    return core.equilibrium(Q, np.ones((nz, ny, nx)), u), solid


def fluid_digest(f, solid):
    """SHA-256 of the fluid cells' values of a (Q, nz, ny, nx) float64 array, in
    (q, z, y, x) order, little-endian."""
    m = ~np.asarray(solid, bool)
    v = np.ascontiguousarray(np.asarray(f, dtype="<f8")[:, m])
    return hashlib.sha256(v.tobytes()).hexdigest()
