"""Checkpointed adjoint of a collide-stream rollout, and its torch.autograd wrapper.

A :class:`Rollout` runs ``steps`` AB-push lattice steps from a fixed initial
state and accumulates a loss over a window of steps
``window = (t0, t1)`` (the state after t steps, t0 <= t <= t1):

* ``"velocity"``: time_weight * sum_x W(x) . u(x, t), W of shape (3, ...);
* ``"energy"``:   time_weight * sum_x W(x) rho |u|^2 / 2, W of shape (...);

with u = (sum c f + F/2) / rho.  The gradient with respect to the per-cell
force field F(x) and porosity (partial bounce-back solid fraction) s(x) comes
from the hand-written adjoint kernel (``lbm_adjoint_step``).  The forward
stores the state every ``checkpoint_every`` steps; the reverse sweep recomputes
each segment from its checkpoint into ``checkpoint_every`` state buffers and
runs the adjoint back through it.  Device memory: (steps / checkpoint_every +
checkpoint_every + 1) population buffers plus three FP64 adjoint buffers.

Device arrays (torch, float64, CUDA) are planar with ``plane`` elements per
component; :meth:`Rollout.to_plane` / :meth:`Rollout.from_plane` convert from
and to (nz, ny, nx) arrays.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _native as N
from .simulation import Simulation

LOSS_KINDS = {"velocity": N.LOSS_VELOCITY, "energy": N.LOSS_ENERGY}


def _vp(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class Rollout:
    def __init__(self, sim: Simulation, steps: int, checkpoint_every: int, loss: str, weight, window,
                 time_weight: float = 1.0):
        if sim.pattern != "ab_push":
            raise ValueError("the adjoint differentiates AB-push rollouts (pattern='ab_push')")
        self.sim = sim
        self.lib = sim.lib
        self.h = sim.h
        self.steps = int(steps)
        self.K = int(checkpoint_every)
        self.kind = LOSS_KINDS[loss]
        self.t0, self.t1 = int(window[0]), int(window[1])
        self.tw = float(time_weight)
        info = sim.info
        self.Q = sim.Q
        self.plane = int(info.plane_stride)
        self.ncell = sim.ncell
        self.buffer_bytes = int(info.buffer_bytes)
        self.dev = torch.device("cuda", sim.cfg.device)
        w = torch.as_tensor(weight, dtype=torch.float64)
        if loss == "velocity":
            self.weight = self.to_plane(w.reshape(3, -1), ncomp=3)
        else:
            self.weight = self.to_plane(w.reshape(1, -1), ncomp=1)
        self.force_field = None
        self.porosity = None
        self._alloc = lambda: torch.empty(self.buffer_bytes, dtype=torch.uint8, device=self.dev)
        self.init_state = self._alloc()
        self._check(self.lib.lbm_copy_state(self.h, _vp(self.init_state), 0))
        nseg = (self.steps + self.K - 1) // self.K
        self.ckpt = [self._alloc() for _ in range(nseg)]
        self.final_state = self._alloc()
        self.seg = None

    # ------------------------------------------------------------ helpers
    def _check(self, st):
        N.check(st, self.h)

    def to_plane(self, a, ncomp):
        """(ncomp, ncell)-shaped data -> (ncomp, plane) float64 device tensor."""
        a = torch.as_tensor(a, dtype=torch.float64).reshape(ncomp, self.ncell)
        out = torch.zeros((ncomp, self.plane), dtype=torch.float64, device=self.dev)
        out[:, :self.ncell] = a.to(self.dev)
        return out

    def from_plane(self, a):
        nz, ny, nx = self.sim.shape
        return a[..., :self.ncell].reshape(a.shape[:-1] + (nz, ny, nx))

    def set_fields(self, force_field=None, porosity=None):
        """force_field (3, ...) and porosity (...) on the grid; None removes."""
        self.force_field = None if force_field is None else self.to_plane(force_field.reshape(3, -1), 3)
        self.porosity = None if porosity is None else self.to_plane(porosity.reshape(1, -1), 1)
        self._check(self.lib.lbm_set_fields_device(self.h, _vp(self.force_field), _vp(self.porosity)))

    def _in_window(self, t):
        return self.t0 <= t <= self.t1

    # ------------------------------------------------------------ forward
    def run_forward(self, store=True) -> float:
        self._check(self.lib.lbm_copy_state(self.h, _vp(self.init_state), 1))
        loss = 0.0
        out = ctypes.c_double(0.0)
        for t in range(self.steps):
            if store and t % self.K == 0:
                self._check(self.lib.lbm_copy_state(self.h, _vp(self.ckpt[t // self.K]), 0))
            self.sim.step(1)
            if self._in_window(t + 1):
                self._check(self.lib.lbm_loss(self.h, None, self.kind, _vp(self.weight), self.tw, ctypes.byref(out)))
                loss += out.value
        if store:
            self._check(self.lib.lbm_copy_state(self.h, _vp(self.final_state), 0))
        self.sim.synchronize()
        return loss

    # ------------------------------------------------------------ adjoint
    def run_backward(self):
        """(grad_force (3, plane), grad_porosity (plane,)) after run_forward(store=True)."""
        Q, P = self.Q, self.plane
        lam_next = torch.zeros((Q, P), dtype=torch.float64, device=self.dev)
        lam = torch.zeros_like(lam_next)
        gF = torch.zeros((3, P), dtype=torch.float64, device=self.dev)
        gS = torch.zeros((P,), dtype=torch.float64, device=self.dev)
        if self.seg is None:
            self.seg = [self._alloc() for _ in range(self.K)]
        T = self.steps
        kind_T = self.kind if self._in_window(T) else N.LOSS_NONE
        # seed: the final state's loss term (its direct force dependence included)
        self._check(self.lib.lbm_adjoint_step(self.h, _vp(self.final_state), None, _vp(lam_next), 0, kind_T,
                                              _vp(self.weight), self.tw, _vp(gF), _vp(gS)))
        nseg = len(self.ckpt)
        for k in reversed(range(nseg)):
            tb, te = k * self.K, min(T, (k + 1) * self.K)
            self._check(self.lib.lbm_copy_state(self.h, _vp(self.ckpt[k]), 1))
            for i in range(te - tb):
                self._check(self.lib.lbm_copy_state(self.h, _vp(self.seg[i]), 0))
                if i < te - tb - 1:
                    self.sim.step(1)
            for t in range(te - 1, tb - 1, -1):
                kind = self.kind if self._in_window(t) else N.LOSS_NONE
                self._check(self.lib.lbm_adjoint_step(self.h, _vp(self.seg[t - tb]), _vp(lam_next), _vp(lam), 1,
                                                      kind, _vp(self.weight), self.tw, _vp(gF), _vp(gS)))
                lam, lam_next = lam_next, lam
        self.sim.synchronize()
        return gF, gS


class RolloutLoss(torch.autograd.Function):
    """loss = RolloutLoss.apply(porosity, force_field, rollout).

    porosity (nz, ny, nx) and force_field (3, nz, ny, nx) are float64 CUDA
    tensors; backward returns dL/dporosity and dL/dforce_field from the
    adjoint."""

    @staticmethod
    def forward(ctx, porosity, force_field, rollout):
        rollout.set_fields(force_field.detach(), porosity.detach())
        loss = rollout.run_forward(store=True)
        ctx.rollout = rollout
        ctx.shape = porosity.shape
        return torch.tensor(loss, dtype=torch.float64, device=porosity.device)

    @staticmethod
    def backward(ctx, grad_out):
        r = ctx.rollout
        gF, gS = r.run_backward()
        return grad_out * r.from_plane(gS), grad_out * r.from_plane(gF), None


def outlet_weight(shape, solid, x_plane, window_len):
    """W for "mean x-velocity on plane x = x_plane over window_len steps":
    1 / (fluid cells in the plane * window_len) on that plane's fluid cells."""
    nz, ny, nx = shape
    w = np.zeros((3, nz, ny, nx))
    fluid = ~np.asarray(solid, bool)[:, :, x_plane]
    w[0, :, :, x_plane] = fluid / (fluid.sum() * window_len)
    return w


def new_rollout(nx, ny, nz, lattice, tau, solid, periodic, steps, checkpoint_every, loss, weight, window,
                storage="f64", force=(0.0, 0.0, 0.0), u0=None, device=0):
    sim = Simulation(nx, ny, nz, lattice=lattice, pattern="ab_push", omega=1.0 / tau, force=force, periodic=periodic,
                     storage=storage, arithmetic="f64" if storage == "f64" else "auto", device=device)
    sim.set_solid(solid)
    sim.init_equilibrium(None, u0)
    return Rollout(sim, steps, checkpoint_every, loss, weight, window)
