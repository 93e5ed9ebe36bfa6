"""Shared test helpers: golden fixture loading and error metrics."""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
PATTERN_NAMES = {0: "aa", 1: "ab_push", 2: "ab_pull"}


def golden_cases():
    """Box / channel cases (reference kernels on a harness geometry)."""
    return sorted(p.stem for p in GOLDEN.glob("*.npz") if not p.stem.startswith(("cylinder_", "sparse_")))


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
