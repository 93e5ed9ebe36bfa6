"""The compact fluid-only layout's host set-up (lbmminiapp_gb300/csrc/
lbm_compact_tiles.hh), built with g++ and checked on the CPU: the fluid
numbering, the odd step's row tiles (at most 32 cells within 255 in x, split
where the span is longer), each tile's row bases and counts, and the kernel's
neighbour formula (row base + the lane's byte count, one below or one past,
the periodic wrap of x at the row ends) against the neighbour's compact index
computed directly, for every fluid cell and direction."""
import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import core
from lbmminiapp_gb300 import workloads

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("g++ not available")
    out = tmp_path_factory.mktemp("ctiles") / "libctiles.so"
    subprocess.run([cxx, "-O2", "-std=c++17", "-shared", "-fPIC", "-I", str(ROOT / "lbmminiapp_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "compact_tiles_check.cpp"), "-o", str(out)], check=True)
    lib = ctypes.CDLL(str(out))
    P, LL = ctypes.c_void_p, ctypes.c_longlong
    lib.compact_tiles_host.argtypes = [ctypes.c_int] * 3 + [P] * 4 + [LL, LL, ctypes.POINTER(LL), ctypes.POINTER(LL)]
    return lib


def build(lib, solid):
    nz, ny, nx = solid.shape
    s = np.ascontiguousarray(solid, dtype=np.uint8)
    cap = int((s == 0).sum()) + 1
    dcell = np.zeros(cap, np.uint32)
    tiles = np.zeros((cap, 20), np.uint32)
    u = np.zeros((cap, 64), np.uint32)
    nf, nt = ctypes.c_longlong(), ctypes.c_longlong()
    rc = lib.compact_tiles_host(nx, ny, nz, s.ctypes.data, dcell.ctypes.data, tiles.ctypes.data, u.ctypes.data,
                                cap, cap, ctypes.byref(nf), ctypes.byref(nt))
    assert rc == 0
    return dcell[:nf.value], tiles[:nt.value], u[:nt.value].reshape(-1, 32, 2)


def check(lib, Q, solid, periodic):
    """Every tile and lane against the mask; returns the number of tiles."""
    nz, ny, nx = solid.shape
    c, opp, _ = core.stencil(Q)
    fluid = solid == 0
    dcell, tiles, u = build(lib, solid)
    assert np.array_equal(dcell, np.flatnonzero(fluid.ravel()))
    cidx = -np.ones(fluid.size, np.int64)
    cidx[dcell] = np.arange(dcell.size)
    cidx = cidx.reshape(nz * ny, nx)
    rows = fluid.reshape(nz * ny, nx)
    count = rows.sum(axis=1)
    rstart = np.concatenate([[0], np.cumsum(count)[:-1]])
    # compact index of the first fluid cell at or after x (past the row's
    # cells: the next row's start)
    first_at = rstart[:, None] + np.concatenate([np.zeros((nz * ny, 1), np.int64),
                                                 np.cumsum(rows, axis=1)], axis=1)[:, :nx + 1]
    seen = 0
    for t, tile in enumerate(tiles):
        b, n, ncell = tile[:9].astype(np.int64), tile[9:18].astype(np.int64), int(tile[18])
        assert 1 <= ncell <= 32
        assert not u[t, ncell:].any()
        i0 = int(b[4])
        r, xa = divmod(int(dcell[i0]), nx)
        y, z = r % ny, r // ny
        nbr = [((y + k // 3 - 1) % ny) + ny * ((z + k % 3 - 1) % nz) for k in range(9)]
        for k in range(9):
            assert b[k] == first_at[nbr[k], xa] and n[k] == count[nbr[k]]
        for lane in range(ncell):
            i = i0 + lane
            rr, x = divmod(int(dcell[i]), nx)
            assert rr == r and 0 <= x - xa <= 255 and i == seen
            seen += 1
            bytes_ = [(int(u[t, lane, j // 4]) >> (8 * (j % 4))) & 0xFF for j in range(8)]
            cnt = bytes_[:4] + [lane] + bytes_[4:]
            N = [int(b[k]) + cnt[k] for k in range(9)]
            for s in range(Q):
                if not c[s].any():
                    continue
                xx, yy, zz = x + c[s, 0], y + c[s, 1], z + c[s, 2]
                outside = any(not periodic[d] and not 0 <= v < m
                              for d, (v, m) in enumerate(((xx, nx), (yy, ny), (zz, nz))))
                if outside or solid[zz % nz, yy % ny, xx % nx]:
                    continue   # blocked: the kernel uses the cell's own slot
                k = (c[s, 1] + 1) * 3 + (c[s, 2] + 1)
                if c[s, 0] == 0:
                    got = N[k]
                elif c[s, 0] < 0:
                    got = N[k] - 1 + (n[k] if x == 0 else 0)
                else:
                    fl = 1 if k == 4 else int(fluid[(z + c[s, 2]) % nz, (y + c[s, 1]) % ny, x])
                    got = N[k] + fl - (n[k] if x == nx - 1 else 0)
                want = cidx[((zz % nz) * ny + yy % ny), xx % nx]
                assert got == want, (t, lane, s)
    assert seen == dcell.size
    return len(tiles)


def sparse_rows(nx, ny, nz, seed):
    rng = np.random.default_rng(seed)
    solid = (rng.random((nz, ny, nx)) < 0.3).astype(np.uint8)
    for z in range(nz):
        row = np.ones(nx, np.uint8)
        x = int(rng.integers(0, 9))
        while x < nx:
            row[x] = 0
            x += int(rng.integers(9, 14))
        solid[z, z % ny] = row
    return solid


@pytest.mark.parametrize("Q", [19, 27])
@pytest.mark.parametrize("name", ["channel_ragged", "periodic_porous", "rows_of_one", "open_x", "sparse_rows",
                                  "spheres"])
def test_row_tiles_and_neighbour_formula(lib, Q, name):
    rng = np.random.default_rng(3)
    if name == "channel_ragged":
        solid = workloads.channel_mask(13, 9, 7) | (rng.random((7, 9, 13)) < 0.12).astype(np.uint8)
        periodic = (1, 0, 1)
    elif name == "periodic_porous":
        solid, periodic = (rng.random((6, 10, 40)) < 0.35).astype(np.uint8), (1, 1, 1)
    elif name == "rows_of_one":
        solid, periodic = (rng.random((6, 8, 1)) < 0.2).astype(np.uint8), (1, 1, 1)
    elif name == "open_x":
        solid, periodic = (rng.random((5, 6, 20)) < 0.15).astype(np.uint8), (0, 1, 1)
    elif name == "sparse_rows":
        solid, periodic = sparse_rows(600, 3, 3, seed=5), (1, 1, 1)
    else:
        solid, _, _ = workloads.sphere_packing(20, 0.35, 3.0, 5.0, seed=5)
        periodic = (1, 1, 1)
    check(lib, Q, solid, periodic)
    if name == "sparse_rows":
        # spans of 32 cells exceed 255 here: some tile holds fewer than 32
        # cells and the next tile continues its row
        dcell, tiles, _ = build(lib, solid)
        nx = solid.shape[2]
        row_of = dcell // nx
        split = [t for t in range(len(tiles) - 1)
                 if tiles[t, 18] < 32 and row_of[tiles[t + 1, 4]] == row_of[tiles[t, 4]]]
        assert split


def test_all_fluid_and_empty_rows(lib):
    for solid in (np.zeros((2, 3, 70), np.uint8), np.ones((2, 3, 5), np.uint8)):
        dcell, tiles, u = build(lib, solid)
        assert dcell.size == int((solid == 0).sum())
        assert len(tiles) == (6 * 3 if not solid.any() else 0)
