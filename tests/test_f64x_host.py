"""F64X collision compiled for the host: precision against the exact IEEE
double collision and the conditions that send a cell to the exact path.
CPU only (nvcc builds host code without a GPU)."""
import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import core

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def f64x(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(nvcc).exists():
        pytest.skip("nvcc not available")
    out = tmp_path_factory.mktemp("f64x") / "libf64x_host.so"
    subprocess.run([nvcc, "-O2", "-std=c++17", "--expt-relaxed-constexpr", "-shared", "-Xcompiler", "-fPIC",
                    "-I", str(ROOT / "lbmminiapp_gb300" / "csrc"), str(ROOT / "tests" / "native" / "f64x_host_check.cu"),
                    "-o", str(out)], check=True)
    lib = ctypes.CDLL(str(out))
    P = ctypes.c_void_p
    lib.f64x_collide_host.argtypes = [ctypes.c_int, P, P, ctypes.c_int, ctypes.c_double, P, ctypes.c_int,
                                      ctypes.c_int, P]
    lib.f64x_collide_host_q27_rolled.argtypes = [P, P, ctypes.c_int, ctypes.c_double, P, ctypes.c_int, ctypes.c_int, P]
    return lib


def collide_exact(Q, f, omega, F, compat=False):
    """Reference BGK + Guo collision (src/kernels/KernelAA_SOA_Base.cpp:186-247), cells along axis 0."""
    c, _, w = core.stencil(Q)
    wf = w.copy()
    if compat and Q == 19:
        wf[18] = 1.0 / 36.0
    rho = f.sum(axis=1)
    v = (f @ c.astype(float) + 0.5 * np.asarray(F)) / rho[:, None]
    vv = 3.0 * (v * v).sum(axis=1)
    fv = 3.0 * (v @ np.asarray(F))
    cu = 3.0 * v @ c.T.astype(float)
    cf = 3.0 * (c.astype(float) @ np.asarray(F))
    eq = w * rho[:, None] * (1.0 + cu + 0.5 * cu * cu - 0.5 * vv[:, None])
    fd = wf * (cf - fv[:, None] + cu * cf)
    return (1.0 - omega) * f + omega * eq + (1.0 - 0.5 * omega) * fd


def random_cells(Q, n, U, neq, seed):
    rng = np.random.default_rng(seed)
    u = rng.uniform(-U, U, (3, n))
    rho = 1.0 + rng.uniform(-0.01, 0.01, n)
    f = core.equilibrium(Q, rho, u).T.copy()
    f *= 1.0 + neq * rng.standard_normal(f.shape)
    return f


def run(lib, Q, f, omega, F, compat=0, force_mode=-1):
    """force_mode: 1 = forcing added after the equilibrium, 2 = folded into it
    (small forces), -1 = the library's choice for this force and omega."""
    f = np.ascontiguousarray(f)
    out = np.empty_like(f)
    fast = np.empty(f.shape[0], np.int32)
    Fa = np.asarray(F, dtype=np.float64)
    lib.f64x_collide_host(Q, f.ctypes.data, out.ctypes.data, f.shape[0], omega, Fa.ctypes.data, compat,
                          force_mode, fast.ctypes.data)
    return out, fast.astype(bool)


@pytest.mark.parametrize("Q", [19, 27])
@pytest.mark.parametrize("omega", [1.0 / 0.55, 1.25, 1.0, 0.7])
@pytest.mark.parametrize("F,mode", [((0.0, 0.0, 0.0), -1), ((1e-5, -2e-6, 3e-6), 1), ((1e-5, -2e-6, 3e-6), 2),
                                    ((1e-3, 5e-4, -2e-4), 2), ((3e-2, -1e-2, 1e-2), 1)])
def test_fast_path_matches_exact_collision(f64x, Q, omega, F, mode):
    f = random_cells(Q, 4000, 0.08, 0.02, seed=Q)
    out, fast = run(f64x, Q, f, omega, F, force_mode=mode)
    assert fast.mean() > 0.99
    ref = collide_exact(Q, f, omega, F)
    err = np.abs(out[fast] - ref[fast]) / np.abs(ref[fast])
    assert err.max() < 2e-13, err.max()        # per step, per population (relative)
    assert np.median(err) < 2e-14


@pytest.mark.parametrize("mode", [1, 2])
def test_compat_rest_weight(f64x, mode):
    f = random_cells(19, 500, 0.05, 0.01, seed=3)
    F = (1e-5, 0.0, 0.0)
    out, fast = run(f64x, 19, f, 1.3, F, compat=1, force_mode=mode)
    ref = collide_exact(19, f, 1.3, F, compat=True)
    assert fast.all()
    assert (np.abs(out - ref) / np.abs(ref)).max() < 2e-13


def test_force_mode_choice(f64x):
    """The folded form is picked only for sum |F_d| <= 0.004 omega; both forms
    give the same results to F64X precision there."""
    f = random_cells(27, 2000, 0.08, 0.02, seed=11)
    for omega, F in ((1.0, (2e-3, 1e-3, 5e-4)), (0.5, (1e-3, 1e-3, 1e-5))):
        auto, fa = run(f64x, 27, f, omega, F)
        one, f1 = run(f64x, 27, f, omega, F, force_mode=1)
        two, f2 = run(f64x, 27, f, omega, F, force_mode=2)
        small = sum(abs(x) for x in F) <= 0.004 * omega
        assert np.array_equal(auto[fa], (two if small else one)[fa])
        assert (fa == f1).all() and (fa == f2).all()
        assert (np.abs(one[fa] - two[fa]) / np.abs(one[fa])).max() < 2e-13


@pytest.mark.parametrize("case", ["zero", "negative", "above_one", "fast_flow", "nan"])
def test_out_of_range_cells_take_the_exact_path(f64x, case):
    f = random_cells(19, 8, 0.02, 0.0, seed=5)
    if case == "zero":
        f[3, 7] = 0.0
    elif case == "negative":
        f[3, 7] = -1e-3
    elif case == "above_one":
        f[3, 18] = 1.5
    elif case == "nan":
        f[3, 2] = np.nan
    else:
        f[3] = core.equilibrium(19, np.ones(1), np.array([[0.15], [0.0], [0.0]]))[:, 0]
    _, fast = run(f64x, 19, f, 1.2, (0, 0, 0))
    assert not fast[3]
    assert fast[[0, 1, 2, 4, 5, 6, 7]].all()


@pytest.mark.parametrize("Q", [19, 27])
@pytest.mark.parametrize("omega", [1.0, 1.0 / 0.6])
def test_slow_flow_momentum_precision(f64x, Q, omega):
    """A slow flow (u ~ 1e-4, as in the reference's cylinder start-up) keeps
    its momentum to double precision: the moment sums become float pairs with
    relative precision, so the per-cell momentum error stays at the level of
    the reference's own double rounding (about 3e-16 rms here, against 1.6e-15
    with a fixed-point conversion of absolute precision 2^-48)."""
    rng = np.random.default_rng(7)
    n = 20000
    u = rng.uniform(-1e-4, 1e-4, (3, n))
    u[0] += 1e-4
    rho = 1.0 + rng.uniform(-1e-4, 1e-4, n)
    f = core.equilibrium(Q, rho, u).T.copy()
    f *= 1.0 + 1e-5 * rng.standard_normal(f.shape)
    F = (1e-6, 0.0, 0.0)
    out, fast = run(f64x, Q, f, omega, F)
    assert fast.all()
    ref = collide_exact(Q, f, omega, F)
    c, _, _ = core.stencil(Q)
    mom = (out - ref) @ c.astype(float)
    assert np.sqrt((mom ** 2).mean()) < 8e-16


def test_result_just_below_a_float_boundary(f64x):
    """A result whose float-pair low part is a tiny negative (here direction
    16: h = 0.0276889801, l = -5.6e-17) rounds toward zero to h's float
    predecessor, and the remainder rounds up to one whole float ulp; that ulp
    must carry into the double pattern.  (Found by a 4-million-cell sweep of
    tau = 0.55 Taylor-Green-like cells, where it cost 6.7e-8 relative.)"""
    cell = [float.fromhex(h) for h in (
        "0x1.ae2c8324d2d6dp-5", "0x1.df4fd961ff843p-5", "0x1.e568aa7948808p-5", "0x1.a8adb322a2eaap-5",
        "0x1.e51683e1d462dp-5", "0x1.a90b4b095a7e1p-5", "0x1.cbe4555e817e2p-6", "0x1.92844aa53813fp-6",
        "0x1.cb7f469f0f6bdp-6", "0x1.92d239a1abce6p-6", "0x1.0025120996eccp-5", "0x1.c035ca2a223b1p-6",
        "0x1.ffd4481221c61p-6", "0x1.c0b3caaa5da2ep-6", "0x1.0336a038a95a6p-5", "0x1.c677903f61c87p-6",
        "0x1.c5a3e4f854109p-6", "0x1.8dc3c88c39b46p-6", "0x1.547e39b6a6ecdp-2")]
    f = np.array([cell])
    out, fast = run(f64x, 19, f, 1.0 / 0.55, (0.0, 0.0, 0.0))
    ref = collide_exact(19, f, 1.0 / 0.55, (0.0, 0.0, 0.0))
    assert fast.all()
    assert (np.abs(out - ref) / np.abs(ref)).max() < 2e-13


@pytest.mark.parametrize("Q", [19, 27])
def test_wide_sweep_of_flow_cells(f64x, Q):
    """Two million cell updates of moderate flows near equilibrium at
    tau = 0.55: every fast-path population within 2e-13 of the exact
    collision."""
    rng = np.random.default_rng(100 + Q)
    n = 2_000_000 // Q
    u = rng.uniform(-0.05, 0.05, (3, n)) + rng.uniform(-1e-3, 1e-3, (3, n))
    f = core.equilibrium(Q, 1.0 + rng.uniform(-1e-3, 1e-3, n), u).T.copy()
    f *= 1.0 + 1e-4 * rng.standard_normal(f.shape)
    out, fast = run(f64x, Q, f, 1.0 / 0.55, (0.0, 0.0, 0.0))
    ref = collide_exact(Q, f, 1.0 / 0.55, (0.0, 0.0, 0.0))
    assert fast.all()
    assert (np.abs(out - ref) / np.abs(ref)).max() < 2e-13


@pytest.mark.parametrize("omega", [1.0 / 0.55, 1.25, 1.0 / 0.6, 0.7])
@pytest.mark.parametrize("F,mode", [((0.0, 0.0, 0.0), -1), ((1e-6, 0.0, 0.0), 2), ((1e-5, -2e-6, 3e-6), 1),
                                    ((1e-3, 5e-4, -2e-4), 2), ((3e-2, -1e-2, 1e-2), 1)])
def test_q27_pair_class_loops_give_the_same_bits(f64x, omega, F, mode):
    """The D3Q27 step kernels run the fast path with its 13 opposite pairs in
    three loops over the pair classes; it must give the unrolled form's bits
    and take the fast path for the same cells (including cells sent to the
    exact path: fast velocities, far from equilibrium)."""
    cells = np.concatenate([random_cells(27, 3000, 0.08, 0.02, seed=7), random_cells(27, 500, 0.3, 0.3, seed=8)])
    want, want_fast = run(f64x, 27, cells, omega, F, force_mode=mode)
    out = np.empty_like(cells)
    fast = np.empty(cells.shape[0], np.int32)
    Fa = np.asarray(F, dtype=np.float64)
    f64x.f64x_collide_host_q27_rolled(cells.ctypes.data, out.ctypes.data, cells.shape[0], omega, Fa.ctypes.data, 0,
                                      mode, fast.ctypes.data)
    assert np.array_equal(fast.astype(bool), want_fast)
    assert want_fast.mean() > 0.5 and not want_fast.all()
    assert np.array_equal(out.view(np.uint64)[want_fast], want.view(np.uint64)[want_fast])
