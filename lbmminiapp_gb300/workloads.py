"""Synthetic inputs of the benchmark configurations (seeded, host side).

* Taylor-Green vortex u = U sin(kx x) cos(ky y) cos(kz z),
  v = -U cos(kx x) sin(ky y) cos(kz z), w = 0, with k = 2 pi / n per axis and
  x, y, z the cell indices;
* uniform velocity noise from a counter-based generator (SplitMix64 keyed by
  seed, cell and component) so every machine produces the same field;
* channel (solid rows y = 0 and y = ny - 1), random sphere packings and
  smoothed porosity fields.
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def splitmix64(x: np.ndarray) -> np.ndarray:
    """SplitMix64 finaliser (Steele, Lea & Flood 2014) on uint64 counters."""
    with np.errstate(over="ignore"):
        z = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
        z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
        z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
        return z ^ (z >> np.uint64(31))


def uniform_noise(shape, seed: int, component: int, amplitude: float) -> np.ndarray:
    """Uniform values in [-amplitude, amplitude) per cell, keyed by
    (seed, cell index, component)."""
    n = int(np.prod(shape))
    cell = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        key = (np.uint64(seed) * np.uint64(0xD1B54A32D192ED03)
               + np.uint64(component) * np.uint64(0x8CB92BA72F3D8DD7)) & _M64
        bits = splitmix64(cell ^ key)
    unit = (bits >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return (amplitude * (2.0 * unit - 1.0)).reshape(shape)


def taylor_green(nx, ny, nz, U=0.05, noise=0.0, seed=0):
    """Velocity field (3, nz, ny, nx) of the 3-D Taylor-Green vortex."""
    kx, ky, kz = 2 * np.pi / nx, 2 * np.pi / ny, 2 * np.pi / nz
    x, y, z = np.arange(nx), np.arange(ny), np.arange(nz)
    u = np.empty((3, nz, ny, nx))
    u[0] = U * (np.cos(kz * z)[:, None, None] * np.cos(ky * y)[None, :, None]) * np.sin(kx * x)[None, None, :]
    u[1] = -U * (np.cos(kz * z)[:, None, None] * np.sin(ky * y)[None, :, None]) * np.cos(kx * x)[None, None, :]
    u[2] = 0.0
    if noise:
        for d in range(3):
            u[d] += uniform_noise((nz, ny, nx), seed, d, noise)
    return u


def channel_mask(nx, ny, nz):
    """Solid rows at y = 0 and y = ny - 1 (half-way walls at y = 0.5 and ny - 1.5)."""
    s = np.zeros((nz, ny, nx), np.uint8)
    s[:, 0, :] = 1
    s[:, ny - 1, :] = 1
    return s


def sphere_packing(n, solid_fraction=0.35, rmin=6.0, rmax=12.0, seed=0, max_tries=200000):
    """Non-overlapping spheres, radius U[rmin, rmax], placed by rejection with
    periodic minimum-image distances until the solid fraction is reached.
    Returns (solid (n,n,n) uint8, centres (k,3), radii (k,))."""
    rng = np.random.default_rng(seed)
    centres, radii = [], []
    solid = np.zeros((n, n, n), bool)
    target = solid_fraction * n ** 3
    count = 0
    tries = 0
    ax = np.arange(n)
    while count < target and tries < max_tries:
        tries += 1
        c = rng.uniform(0, n, 3)
        r = rng.uniform(rmin, rmax)
        ok = True
        for c2, r2 in zip(centres, radii):
            d = np.abs(c - c2)
            d = np.minimum(d, n - d)
            if np.sqrt((d * d).sum()) < r + r2:
                ok = False
                break
        if not ok:
            continue
        centres.append(c)
        radii.append(r)
        lo = np.floor(c - r).astype(int)
        hi = np.ceil(c + r).astype(int) + 1
        zi = ax.take(range(lo[2], hi[2]), mode="wrap")
        yi = ax.take(range(lo[1], hi[1]), mode="wrap")
        xi = ax.take(range(lo[0], hi[0]), mode="wrap")
        dz = np.arange(lo[2], hi[2]) - c[2]
        dy = np.arange(lo[1], hi[1]) - c[1]
        dx = np.arange(lo[0], hi[0]) - c[0]
        inside = (dz[:, None, None] ** 2 + dy[None, :, None] ** 2 + dx[None, None, :] ** 2) <= r * r
        sub = solid[np.ix_(zi, yi, xi)]
        sub |= inside
        solid[np.ix_(zi, yi, xi)] = sub
        count = int(solid.sum())
    return solid.astype(np.uint8), np.array(centres), np.array(radii)


def smoothed_porosity(shape, sigma=3.0, seed=0, mean=0.15, spread=0.1):
    """Seeded N(0,1) noise smoothed by a periodic Gaussian of width sigma,
    normalised to unit variance, mapped affinely to mean + spread * z and
    clipped to [0, 1]."""
    rng = np.random.default_rng(seed)
    noise = rng.standard_normal(shape)
    freqs = [np.fft.fftfreq(n) for n in shape]
    k2 = sum(np.meshgrid(*[(2 * np.pi * f) ** 2 for f in freqs], indexing="ij"))
    smooth = np.real(np.fft.ifftn(np.fft.fftn(noise) * np.exp(-0.5 * sigma * sigma * k2)))
    smooth = (smooth - smooth.mean()) / smooth.std()
    return np.clip(mean + spread * smooth, 0.0, 1.0)
