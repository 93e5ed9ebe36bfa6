"""Compact fluid-only layout on the GPU (lbm_sparse_*): the reference's own
buffers, fluid order and adjacency list for its cylinder, stepped by the CUDA
kernels and compared with the reference's final raw buffer
(tests/golden/sparse_*.npz, made by tests/golden/make_golden.py from the
reference's app flow with the Base kernels).  Exact FP64 arithmetic must be
bit-identical; F64X within 1e-10 relative."""
import numpy as np
import pytest

from _helpers import load_golden, rel_err, sparse_cases
from lbmminiapp_gb300 import cylinder, sparse

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

PATTERNS = {(1, 0): "aa", (0, 0): "ab_push", (0, 1): "ab_pull"}


def weights(Q):
    if Q == 19:
        table = {0: 1.0 / 3.0, 1: 1.0 / 18.0, 2: 1.0 / 36.0}
    else:
        table = {0: 8.0 / 27.0, 1: 2.0 / 27.0, 2: 1.0 / 54.0, 3: 1.0 / 216.0}
    c = sparse.velocities(Q)
    return np.array([table[int(k)] for k in (c * c).sum(axis=1)])


def run_case(g, arithmetic, adjacency=None, chunks=1):
    """Rest start (every slot s holds w_s, as PropagationAA/AB::initialize
    writes it), g['steps'] steps; returns the final raw buffer [Q, nfluid]."""
    Q = int(g["Q"])
    adj = g["adjacency"] if adjacency is None else adjacency
    n = adj.shape[1]
    pattern = PATTERNS[(int(g["prop_pattern"]), int(g["pull"]))]
    f0 = np.repeat(weights(Q)[:, None], n, axis=1)
    bufs = [torch.tensor(f0, dtype=torch.float64, device="cuda") for _ in range(1 if pattern == "aa" else 2)]
    with sparse.SparseKernels(adj, lattice=Q, pattern=pattern, omega=float(g["omega"]),
                              force=(float(g["gx"]), 0.0, 0.0), arithmetic=arithmetic) as k:
        if chunks == 1:
            out = k.run(bufs, int(g["steps"]))
        else:
            # border/bulk-style range calls (PropagationAA.cpp:173-174)
            edges = np.linspace(0, n, chunks + 1).astype(int)
            src = bufs[0]
            tgt = bufs[1] if len(bufs) > 1 else None
            for t in range(int(g["steps"])):
                for a, b in zip(edges[:-1], edges[1:]):
                    if pattern == "aa":
                        (k.timestep_even_force if t % 2 == 0 else k.timestep_odd_force)(src, int(a), int(b - a))
                    else:
                        k.timestep_force(src, tgt, int(a), int(b - a))
                if tgt is not None:
                    src, tgt = tgt, src
            out = src
        torch.cuda.synchronize()
        return out.cpu().numpy()


@pytest.mark.parametrize("name", sparse_cases())
def test_exact_arithmetic_is_bit_identical_to_reference(gpu, name):
    g = load_golden(name)
    out = run_case(g, "f64")
    assert np.array_equal(out, g["raw_final"]), rel_err(out, g["raw_final"])


@pytest.mark.parametrize("name", sparse_cases())
def test_f64x_within_1e10_of_reference(gpu, name):
    g = load_golden(name)
    out = run_case(g, "f64x")
    assert rel_err(out, g["raw_final"]) <= 1e-10


@pytest.mark.parametrize("arithmetic", ["f64", "f64x"])
@pytest.mark.parametrize("name", ["sparse_q19_aa_cylinder", "sparse_q19_ab_pull_cylinder",
                                  "sparse_q27_aa_cylinder"])
def test_range_calls_compose(gpu, name, arithmetic):
    """Border/bulk-style range calls (ranges not a multiple of the 32-point
    tiles of the pipelined F64X kernel) equal one full-range call."""
    g = load_golden(name)
    if arithmetic == "f64" and name in sparse_cases():
        want = g["raw_final"]
    else:
        want = run_case(g, arithmetic)
    assert np.array_equal(run_case(g, arithmetic, chunks=3), want)


@pytest.mark.parametrize("arithmetic", ["f64", "f64x"])
@pytest.mark.parametrize("name", ["sparse_q19_aa_cylinder", "sparse_q19_ab_push_cylinder"])
def test_any_fluid_order(gpu, name, arithmetic):
    """The same geometry in a shuffled fluid order gives the shuffled result."""
    g = load_golden(name)
    adj = g["adjacency"].astype(np.int64)
    Q, n = adj.shape
    perm = np.random.default_rng(5).permutation(n)
    inv = np.empty(n, np.int64)
    inv[perm] = np.arange(n)
    s_part, j_part = np.divmod(adj[:, perm], n)
    adj_p = (s_part * n + inv[j_part]).astype(np.int32)
    out = run_case(g, arithmetic, adjacency=adj_p)
    want = g["raw_final"] if arithmetic == "f64" else run_case(g, arithmetic)
    assert np.array_equal(out, want[:, perm])


@pytest.mark.parametrize("arithmetic", ["f64", "f64x"])
@pytest.mark.parametrize("Q,pattern", [(19, "aa"), (19, "ab_push"), (19, "ab_pull"), (27, "aa"), (27, "ab_pull")])
def test_matches_dense_layout_on_larger_cylinder(gpu, Q, pattern, arithmetic):
    """build_adjacency + the compact kernels against the dense-layout path
    (link words) on a size-1 cylinder: the same populations bit for bit, in
    either arithmetic (both layouts run the same collision)."""
    import lbmminiapp_gb300 as lbm
    dims, solid = cylinder(1.0)
    nx, ny, nz = dims
    cells, adj = sparse.build_adjacency(solid, (1, 0, 0), pattern, Q)
    omega, gx, steps = 1.0 / 0.6, 1e-5, 9
    with lbm.Simulation(nx, ny, nz, lattice=Q, pattern=pattern, omega=omega, force=(gx, 0, 0),
                        periodic=(1, 0, 0), arithmetic=arithmetic) as sim:
        sim.set_solid(solid)
        sim.init_equilibrium(None, None)
        sim.step(steps)
        dense = sim.get_populations("raw").reshape(Q, -1)[:, cells]
    g = dict(Q=Q, prop_pattern=1 if pattern == "aa" else 0, pull=int(pattern == "ab_pull"), omega=omega,
             gx=gx, steps=steps, adjacency=adj)
    out = run_case(g, arithmetic)
    assert np.array_equal(out, dense)


@pytest.mark.parametrize("Q,pattern", [(19, "aa"), (19, "ab_pull"), (27, "aa"), (27, "ab_push")])
def test_matches_dense_layout_with_tile_feed(gpu, Q, pattern):
    """The same comparison in F64X on a size-4 cylinder (about 1.15 million
    fluid points): at least 16 tiles per warp, so both layouts' persistent
    kernels take their tiles from the tile feed after the fixed first round,
    over 9 steps (each launch re-arms the feed's counters for the next)."""
    import lbmminiapp_gb300 as lbm
    dims, solid = cylinder(4.0)
    nx, ny, nz = dims
    cells, adj = sparse.build_adjacency(solid, (1, 0, 0), pattern, Q)
    assert adj.shape[1] >= 16 * 32 * 152 * 12   # tiles per warp of the 12-warp-per-SM kernel
    omega, gx, steps = 1.0 / 0.6, 1e-5, 9
    with lbm.Simulation(nx, ny, nz, lattice=Q, pattern=pattern, omega=omega, force=(gx, 0, 0),
                        periodic=(1, 0, 0), arithmetic="f64x") as sim:
        sim.set_solid(solid)
        sim.init_equilibrium(None, None)
        sim.step(steps)
        dense = sim.get_populations("raw").reshape(Q, -1)[:, cells]
    g = dict(Q=Q, prop_pattern=1 if pattern == "aa" else 0, pull=int(pattern == "ab_pull"), omega=omega,
             gx=gx, steps=steps, adjacency=adj)
    out = run_case(g, "f64x")
    assert np.array_equal(out, dense)


def test_errors_are_reported(gpu):
    g = load_golden("sparse_q19_aa_cylinder")
    n = g["adjacency"].shape[1]
    buf = torch.zeros((19, n), dtype=torch.float64, device="cuda")
    with sparse.SparseKernels(g["adjacency"], lattice=19, pattern="aa") as k:
        with pytest.raises(lbm_error()) as e:
            k.timestep_force(buf, buf)
        assert e.value.status == 6
        with pytest.raises(lbm_error()) as e:
            k.timestep_even_force(buf, 0, n + 1)
        assert e.value.status == 1
    bad = g["adjacency"].copy()
    bad[3, 5] = 19 * n
    with pytest.raises(lbm_error()):
        sparse.SparseKernels(bad, lattice=19, pattern="aa")


def lbm_error():
    from lbmminiapp_gb300 import LBMError
    return LBMError
