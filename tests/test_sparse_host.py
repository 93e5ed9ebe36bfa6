"""Compact-layout host logic: build_adjacency reproduces the adjacency list
the reference's own GeometryAAAB::setupAdjacency built for its cylinder
(src/geometries/GeometryAAAB.cpp:18-124), from the committed fixtures.  CPU
only."""
import numpy as np
import pytest

from _helpers import load_golden, sparse_cases
from lbmminiapp_gb300 import cylinder, sparse

PATTERNS = {(1, 0): "aa", (0, 0): "ab_push", (0, 1): "ab_pull"}


def reference_order(g, solid):
    """Permutation taking build_adjacency's x-fastest fluid list to the
    reference's sorted fluid list."""
    nz, ny, nx = solid.shape
    pts = g["fluid_pts"].astype(np.int64)
    ref_cells = pts[:, 0] + nx * (pts[:, 1] + ny * pts[:, 2])
    sorted_cells = np.flatnonzero(~solid.astype(bool).ravel())
    order = np.searchsorted(sorted_cells, ref_cells)
    assert np.array_equal(sorted_cells[order], ref_cells)
    return order


@pytest.mark.parametrize("name", sparse_cases())
def test_build_adjacency_matches_reference(name):
    g = load_golden(name)
    dims, solid = cylinder(0.25)
    assert tuple(g["dims"]) == dims
    order = reference_order(g, solid)
    pattern = PATTERNS[(int(g["prop_pattern"]), int(g["pull"]))]
    # one rank: only the pipe axis x wraps (GeometryAAAB.cpp:56-66)
    cells, adj = sparse.build_adjacency(solid, periodic=(1, 0, 0), pattern=pattern, lattice=int(g["Q"]),
                                        order=order)
    assert adj.dtype == np.int32
    assert np.array_equal(adj, g["adjacency"])


def test_build_adjacency_any_order_is_consistent():
    """A permuted fluid list gives the permuted map of the same streaming."""
    rng = np.random.default_rng(3)
    solid = (rng.random((5, 6, 7)) < 0.3).astype(np.uint8)
    cells, adj = sparse.build_adjacency(solid, (1, 1, 0), "aa", 27)
    n = cells.size
    perm = rng.permutation(n)
    cells_p, adj_p = sparse.build_adjacency(solid, (1, 1, 0), "aa", 27, order=perm)
    assert np.array_equal(cells_p, cells[perm])
    inv = np.empty(n, np.int64)
    inv[perm] = np.arange(n)
    # element index n*s' + j in the original order -> n*s' + inv[j] in the permuted one
    s_part, j_part = np.divmod(adj[:, perm].astype(np.int64), n)
    assert np.array_equal(adj_p, (s_part * n + inv[j_part]).astype(np.int32))
