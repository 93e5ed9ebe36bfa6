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


def _wrapped_ball(n, c, r, ax):
    """Index grid (np.ix_) of the periodic box around a ball and the ball's
    squared cell-centre distances on it."""
    lo = np.floor(c - r).astype(int)
    hi = np.ceil(c + r).astype(int) + 1
    g = np.ix_(ax.take(range(lo[2], hi[2]), mode="wrap"), ax.take(range(lo[1], hi[1]), mode="wrap"),
               ax.take(range(lo[0], hi[0]), mode="wrap"))
    dz = np.arange(lo[2], hi[2]) + 0.5 - c[2]
    dy = np.arange(lo[1], hi[1]) + 0.5 - c[1]
    dx = np.arange(lo[0], hi[0]) + 0.5 - c[0]
    return g, dz[:, None, None] ** 2 + dy[None, :, None] ** 2 + dx[None, None, :] ** 2


def sphere_packing(n, solid_fraction=0.35, rmin=6.0, rmax=12.0, seed=0, max_tries=5000000, batch=4096):
    """Non-overlapping spheres of radius U[rmin, rmax] in a periodic n^3 box,
    placed by seeded random sequential addition (minimum-image distances)
    until the solid fraction is reached or max_tries candidates were drawn.
    A cell is solid when its centre lies inside a sphere.

    Candidates are drawn in batches and tested in draw order, so the packing
    is the one a one-at-a-time loop over the same random stream gives.  Two
    filters make the test cheap: a mask of cells whose centre lies within
    r_k + rmin - sqrt(3)/2 of a placed sphere k (a candidate centred in such a
    cell overlaps sphere k whatever its radius), then the exact test against
    the spheres in the 27 neighbouring bins of a periodic cell list (edge >=
    2 rmax).  Returns (solid (n,n,n) uint8, centres (k,3), radii (k,))."""
    if n < 2 * (rmax + rmin) + 4:
        raise ValueError("sphere_packing needs n >= 2 (rmax + rmin) + 4")
    rng = np.random.default_rng(seed)
    nb = max(1, int(n // (2 * rmax)))
    edge = n / nb
    binidx = np.full((nb ** 3, 8), -1, np.int64)
    bincnt = np.zeros(nb ** 3, np.int64)
    C = np.empty((1024, 3))
    R = np.empty(1024)
    k = 0
    solid = np.zeros((n, n, n), bool)
    blocked = np.zeros((n, n, n), bool)
    target = int(round(solid_fraction * n ** 3))
    count = 0
    tries = 0
    ax = np.arange(n)
    off = np.array([(a, b, c) for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)])
    margin = rmin - np.sqrt(3.0) / 2
    while count < target and tries < max_tries:
        cs = rng.uniform(0, n, (batch, 3))
        rs = rng.uniform(rmin, rmax, batch)
        bs = (cs // edge).astype(np.int64) % nb
        ci = np.minimum(cs.astype(np.int64), n - 1)
        sel = np.flatnonzero(~blocked[ci[:, 2], ci[:, 1], ci[:, 0]])
        # exact test against the spheres placed before this batch
        nbv = (bs[sel, None, :] + off[None]) % nb
        idx = binidx[(nbv[..., 0] * nb + nbv[..., 1]) * nb + nbv[..., 2]].reshape(len(sel), -1)
        valid = idx >= 0
        ii = np.where(valid, idx, 0)
        d = np.abs(C[ii] - cs[sel, None, :])
        d = np.minimum(d, n - d)
        hit = valid & ((d * d).sum(-1) < (R[ii] + rs[sel, None]) ** 2)
        free = np.zeros(batch, bool)
        free[sel] = ~hit.any(1)
        base = tries
        tries = min(base + batch, max_tries)
        start = k
        for j in np.flatnonzero(free[:tries - base]):
            c, r = cs[j], rs[j]
            if k > start:   # against the spheres placed earlier in this batch
                dd = np.abs(C[start:k] - c)
                dd = np.minimum(dd, n - dd)
                if ((dd * dd).sum(1) < (R[start:k] + r) ** 2).any():
                    continue
            if k == len(R):
                C = np.concatenate([C, np.empty_like(C)])
                R = np.concatenate([R, np.empty_like(R)])
            C[k], R[k] = c, r
            b = (bs[j, 0] * nb + bs[j, 1]) * nb + bs[j, 2]
            if bincnt[b] == binidx.shape[1]:
                binidx = np.concatenate([binidx, np.full_like(binidx, -1)], 1)
            binidx[b, bincnt[b]] = k
            bincnt[b] += 1
            k += 1
            g, d2 = _wrapped_ball(n, c, r, ax)
            sub = solid[g]
            inside = d2 <= r * r
            count += int((inside & ~sub).sum())
            solid[g] = sub | inside
            g, d2 = _wrapped_ball(n, c, r + margin, ax)
            blocked[g] |= d2 < (r + margin) ** 2
            if count >= target:
                tries = base + j + 1
                break
    return solid.astype(np.uint8), C[:k].copy(), R[:k].copy()


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
