"""Adjoint gradients (no reference counterpart) against FP64 central finite
differences.

Gradient error: max_i |g_adj(i) - g_fd(i)| / max_i |g_fd(i)| over the probed
cells.  Small cases: <= 1e-6.  The porous channel (128 x 64 x 64, D3Q19,
tau = 0.7, porosity from Gaussian noise smoothed with sigma = 3 and clipped,
per-cell force g_x = 1e-5, 500 steps, loss = mean u_x on the plane x = Nx-1 over
steps 451-500, checkpoint every 50, eps = 1e-4 at 16 seeded fluid cells):
<= 1e-4 with the FP64 and with the FP32-storage forward.
"""
import numpy as np
import pytest

from lbmminiapp_gb300 import workloads

pytestmark = pytest.mark.gpu


def make_case(Q, nx, ny, nz, tau, steps, K, loss, window, storage="f64", seed=0, gx=1e-5):
    import torch
    from lbmminiapp_gb300.adjoint import new_rollout, outlet_weight
    solid = workloads.channel_mask(nx, ny, nz)
    if loss == "velocity":
        weight = outlet_weight((nz, ny, nx), solid, nx - 1, window[1] - window[0] + 1)
    else:
        weight = (~solid.astype(bool)).astype(float) / ((~solid.astype(bool)).sum() * (window[1] - window[0] + 1))
    r = new_rollout(nx, ny, nz, Q, tau, solid, (1, 0, 1), steps, K, loss, weight, window, storage=storage)
    poro = workloads.smoothed_porosity((nz, ny, nx), sigma=3.0, seed=seed, mean=0.1, spread=0.1)
    force = np.zeros((3, nz, ny, nx))
    force[0] = gx
    rng = np.random.default_rng(seed + 1)
    force[1] = 1e-6 * rng.standard_normal((nz, ny, nx))
    dev = torch.device("cuda")
    return r, solid, torch.tensor(poro, device=dev), torch.tensor(force, device=dev)


def fd_gradients(r, poro, force, cells, eps=1e-4, eps_f=None):
    """Central differences of the loss w.r.t. porosity (step eps) and F_x (step
    eps_f, default eps) at cells."""
    eps_f = eps if eps_f is None else eps_f
    gs, gf = [], []
    for (z, y, x) in cells:
        vals = []
        for which in ("s", "f"):
            out = []
            for sgn in (+1, -1):
                p2, f2 = poro.clone(), force.clone()
                if which == "s":
                    p2[z, y, x] += sgn * eps
                else:
                    f2[0, z, y, x] += sgn * eps_f
                r.set_fields(f2, p2)
                out.append(r.run_forward(store=False))
            vals.append((out[0] - out[1]) / (2 * (eps if which == "s" else eps_f)))
        gs.append(vals[0])
        gf.append(vals[1])
    return np.array(gs), np.array(gf)


def pick_cells(solid, n, seed):
    rng = np.random.default_rng(seed)
    fluid = np.argwhere(~solid.astype(bool))
    return [tuple(fluid[i]) for i in rng.choice(len(fluid), n, replace=False)]


def grad_err(adj, fd):
    return float(np.abs(adj - fd).max() / np.abs(fd).max())


@pytest.mark.parametrize("Q", [19, 27])
@pytest.mark.parametrize("loss", ["velocity", "energy"])
def test_adjoint_matches_fd_small(gpu, Q, loss):
    r, solid, poro, force = make_case(Q, 20, 12, 10, 0.7, 24, 8, loss, (20, 24), seed=Q)
    r.set_fields(force, poro)
    r.run_forward(store=True)
    gF, gS = r.run_backward()
    gS = r.from_plane(gS).cpu().numpy()
    gFx = r.from_plane(gF)[0].cpu().numpy()
    cells = pick_cells(solid, 6, seed=Q)
    # the energy loss is quadratic in the force (g_x = 1e-5): a force step of
    # 1e-4 would put O(eps^2) truncation above the bound, so it uses 1e-6
    fd_s, fd_f = fd_gradients(r, poro, force, cells, eps=1e-4, eps_f=1e-6 if loss == "energy" else 1e-4)
    adj_s = np.array([gS[c] for c in cells])
    adj_f = np.array([gFx[c] for c in cells])
    assert grad_err(adj_s, fd_s) < 1e-6, (adj_s, fd_s)
    assert grad_err(adj_f, fd_f) < 1e-6, (adj_f, fd_f)


@pytest.mark.parametrize("loss", ["velocity", "energy"])
def test_adjoint_window_from_initial_state(gpu, loss):
    """A loss window that starts at t = 0 counts the initial state in the
    forward loss and in the adjoint alike."""
    r, solid, poro, force = make_case(19, 16, 10, 8, 0.7, 10, 4, loss, (0, 6), seed=9)
    r.set_fields(force, poro)
    r.run_forward(store=True)
    gF, gS = r.run_backward()
    gS = r.from_plane(gS).cpu().numpy()
    gFx = r.from_plane(gF)[0].cpu().numpy()
    cells = pick_cells(solid, 5, seed=4)
    fd_s, fd_f = fd_gradients(r, poro, force, cells, eps=1e-4, eps_f=1e-6 if loss == "energy" else 1e-4)
    assert grad_err(np.array([gS[c] for c in cells]), fd_s) < 1e-6
    assert grad_err(np.array([gFx[c] for c in cells]), fd_f) < 1e-6


def test_autograd_function_matches_run_backward(gpu):
    import torch
    from lbmminiapp_gb300.adjoint import RolloutLoss
    r, solid, poro, force = make_case(19, 16, 10, 8, 0.8, 12, 4, "velocity", (10, 12), seed=3)
    p = poro.clone().requires_grad_(True)
    f = force.clone().requires_grad_(True)
    loss = RolloutLoss.apply(p, f, r)
    loss.backward()
    r.set_fields(force, poro)
    r.run_forward(store=True)
    gF, gS = r.run_backward()
    assert torch.allclose(p.grad, r.from_plane(gS), rtol=1e-12, atol=0)
    assert torch.allclose(f.grad, r.from_plane(gF), rtol=1e-12, atol=0)
    assert float(loss.detach()) > 0


@pytest.mark.parametrize("storage", ["f64", "f32"])
def test_porous_channel_adjoint(gpu, parity_record, storage):
    """C4: D3Q19 AA 128x64x64 channel, smoothed porosity, gx 1e-5, tau 0.7,
    500 steps, checkpoints every 50; loss = mean u_x on x = 127 over steps
    451-500.  The adjoint gradients with respect to porosity and the force
    field agree with FP64 central differences (eps 1e-4) at 16 seeded fluid
    cells within 1e-4 relative, for FP64 and for FP32 storage (the FP32 form
    is the configuration's own)."""
    nx, ny, nz = 128, 64, 64
    r, solid, poro, force = make_case(19, nx, ny, nz, 0.7, 500, 50, "velocity", (451, 500), storage=storage,
                                      seed=42)
    r.set_fields(force, poro)
    loss = r.run_forward(store=True)
    gF, gS = r.run_backward()
    gS = r.from_plane(gS).cpu().numpy()
    gFx = r.from_plane(gF)[0].cpu().numpy()
    cells = pick_cells(solid, 16, seed=7)
    # FP64 central differences with an FP64 forward
    ref, _, _, _ = make_case(19, nx, ny, nz, 0.7, 500, 50, "velocity", (451, 500), storage="f64", seed=42)
    fd_s, fd_f = fd_gradients(ref, poro, force, cells, eps=1e-4)
    adj_s = np.array([gS[c] for c in cells])
    adj_f = np.array([gFx[c] for c in cells])
    es, ef = grad_err(adj_s, fd_s), grad_err(adj_f, fd_f)
    parity_record(f"porous channel adjoint ({storage} storage) vs FP64 central differences",
                  {"porosity": es, "force": ef})
    assert loss > 0
    assert es < 1e-4 and ef < 1e-4


def _grads(r, poro, force):
    r.set_fields(force, poro)
    r.run_forward(store=True)
    gF, gS = r.run_backward()
    return gF.cpu().numpy(), gS.cpu().numpy()


def test_multilevel_checkpoints_give_the_same_gradient(gpu):
    """Recomputing through nested checkpoints replays the same forward states,
    so the gradients are bit-identical to single-level checkpointing."""
    r, solid, poro, force = make_case(19, 20, 12, 10, 0.7, 25, 8, "velocity", (20, 25), seed=5)
    ref = _grads(r, poro, force)
    for strides in [(8, 3), (9, 4, 2), (25, 5, 1)]:
        r.strides = strides
        r.K = strides[0]
        r.ckpt = [r.init_state] + [r._alloc() for _ in range((r.steps + r.K - 1) // r.K - 1)]
        r._pools = {}
        got = _grads(r, poro, force)
        assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1]), strides


@pytest.mark.parametrize("Q", [19, 27])
@pytest.mark.parametrize("storage", ["f64", "f16"])
def test_f32_adjoint_close_to_f64_adjoint(gpu, Q, storage):
    """The FP32 adjoint against the FP64 adjoint over the same forward states:
    relative max error <= 1e-4 for both gradients."""
    r, solid, poro, force = make_case(Q, 20, 12, 10, 0.7, 40, 8, "velocity", (30, 40), storage=storage, seed=Q)
    g64 = _grads(r, poro, force)
    r.adjoint = "f32"
    g32 = _grads(r, poro, force)
    fluid = ~solid.astype(bool)
    for a, b in ((g32[1], g64[1]), (g32[0][0], g64[0][0])):
        a, b = r.from_plane(torch_t(a)).numpy()[fluid], r.from_plane(torch_t(b)).numpy()[fluid]
        assert np.abs(a - b).max() <= 1e-4 * np.abs(b).max()


def torch_t(a):
    import torch
    return torch.from_numpy(a)
