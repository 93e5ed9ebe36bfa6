"""Checkpointed adjoint of a collide-stream rollout, and its torch.autograd wrapper.

A :class:`Rollout` runs ``steps`` AB-push lattice steps from a fixed initial
state and accumulates a loss over a window of steps
``window = (t0, t1)`` (the state after t steps, t0 <= t <= t1, with
0 <= t0 <= t1 <= steps; t = 0 is the initial state):

* ``"velocity"``: time_weight * sum_x W(x) . u(x, t), W of shape (3, ...);
* ``"energy"``:   time_weight * sum_x W(x) rho |u|^2 / 2, W of shape (...);

with u = (sum c f + F/2) / rho.  The gradient with respect to the per-cell
force field F(x) and porosity (partial bounce-back solid fraction) s(x) comes
from the hand-written adjoint kernel: ``lbm_adjoint_step`` (FP64) or
``lbm_adjoint_step_f32`` (adjoint state and arithmetic in FP32, gradients
accumulated in FP64), chosen by ``adjoint="f64" | "f32"``.

Checkpointing is multi-level.  ``checkpoint_every`` is one stride S_0 or a
decreasing tuple (S_0, S_1, ..., S_{L-1}).  The forward stores the state at
every multiple of S_0.  The reverse sweep takes the level-0 segments last to
first; a segment of level l < L is recomputed from its checkpoint, storing the
state at every S_{l+1}-th step (level l+1 checkpoints), and its sub-segments
are reversed the same way; a segment of level L (at most S_{L-1} steps) is
recomputed storing every state and the adjoint runs back through it.  State
buffers held at once: ceil(steps / S_0) + sum_l (ceil(S_{l-1} / S_l) - 1) +
S_{L-1} - 1 + 1 (the final state), plus two adjoint buffers; each level of
checkpoints costs one more forward pass in recomputation.

Device arrays (torch, float64, CUDA) are planar with ``plane`` elements per
component; :meth:`Rollout.to_plane` / :meth:`Rollout.from_plane` convert from
and to (nz, ny, nx) arrays.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _native as N
from .simulation import Simulation

LOSS_KINDS = {"velocity": N.LOSS_VELOCITY, "energy": N.LOSS_ENERGY}


def _vp(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def checkpoint_buffers(steps, strides):
    """State buffers a rollout of ``steps`` with these checkpoint strides holds
    at once (the final state's included, the handle's own not)."""
    strides = (strides,) if isinstance(strides, int) else tuple(strides)
    n = math.ceil(steps / strides[0]) + max(1, strides[-1] - 1)
    for a, b in zip(strides[:-1], strides[1:]):
        n += math.ceil(a / b) - 1
    return n


class Rollout:
    def __init__(self, sim: Simulation, steps: int, checkpoint_every, loss: str, weight, window,
                 time_weight: float = 1.0, adjoint: str = "f64", device=None):
        if sim.pattern != "ab_push":
            raise ValueError("the adjoint differentiates AB-push rollouts (pattern='ab_push')")
        if adjoint not in ("f64", "f32"):
            raise ValueError("adjoint must be 'f64' or 'f32'")
        strides = (checkpoint_every,) if isinstance(checkpoint_every, int) else tuple(checkpoint_every)
        if not strides or any(int(a) <= int(b) for a, b in zip(strides[:-1], strides[1:])) or int(strides[-1]) < 1:
            raise ValueError("checkpoint strides must be positive and strictly decreasing")
        self.sim = sim
        self.lib = sim.lib
        self.h = sim.h
        self.steps = int(steps)
        self.strides = tuple(int(v) for v in strides)
        self.K = self.strides[0]
        self.adjoint = adjoint
        self.kind = LOSS_KINDS[loss]
        self.t0, self.t1 = int(window[0]), int(window[1])
        if not 0 <= self.t0 <= self.t1 <= self.steps:
            raise ValueError(f"loss window {window} must satisfy 0 <= t0 <= t1 <= steps = {self.steps}")
        self.tw = float(time_weight)
        info = sim.info
        self.Q = sim.Q
        self.plane = int(info.plane_stride)
        self.ncell = sim.ncell
        self.buffer_bytes = int(info.buffer_bytes)
        self.dev = torch.device("cuda", sim.cfg.device) if device is None else torch.device(device)
        w = torch.as_tensor(weight, dtype=torch.float64)
        if loss == "velocity":
            self.weight = self.to_plane(w.reshape(3, -1), ncomp=3)
        else:
            self.weight = self.to_plane(w.reshape(1, -1), ncomp=1)
        self.force_field = None
        self.porosity = None
        # the initial state is the first level-0 checkpoint
        self.init_state = self._alloc()
        self._check(self.lib.lbm_copy_state(self.h, _vp(self.init_state), 0))
        nseg = (self.steps + self.K - 1) // self.K
        self.ckpt = [self.init_state] + [self._alloc() for _ in range(nseg - 1)]
        self.final_state = self._alloc()
        self._pools = {}
        self._torch_done()

    # ------------------------------------------------------------ helpers
    def _alloc(self):
        return torch.empty(self.buffer_bytes, dtype=torch.uint8, device=self.dev)

    def release(self):
        """Drop every state buffer (checkpoints, recomputation pools, the
        initial and final states); the rollout cannot run afterwards."""
        self.ckpt = []
        self._pools = {}
        self.init_state = self.final_state = None

    def _check(self, st):
        N.check(st, self.h)

    def _torch_done(self):
        """Wait for torch's work on this device (fills of buffers the handle's
        kernels read or accumulate into): the handle may run on another
        stream than torch's current one."""
        if self.dev.type == "cuda":
            torch.cuda.current_stream(self.dev).synchronize()

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
        self._torch_done()
        self._check(self.lib.lbm_set_fields_device(self.h, _vp(self.force_field), _vp(self.porosity)))

    def _in_window(self, t):
        return self.t0 <= t <= self.t1

    def _pool(self, level, n):
        pool = self._pools.setdefault(level, [])
        while len(pool) < n:
            pool.append(self._alloc())
        return pool[:n]

    def _save(self, buf):
        self._check(self.lib.lbm_copy_state(self.h, _vp(buf), 0))

    def _load(self, buf):
        self._check(self.lib.lbm_copy_state(self.h, _vp(buf), 1))

    # ------------------------------------------------------------ forward
    def run_forward(self, store=True) -> float:
        self._load(self.init_state)
        loss = 0.0
        out = ctypes.c_double(0.0)
        if self._in_window(0):
            # the initial state's own term (its direct force dependence is
            # differentiated by the adjoint step at t = 0)
            self._check(self.lib.lbm_loss(self.h, None, self.kind, _vp(self.weight), self.tw, ctypes.byref(out)))
            loss += out.value
        for t in range(self.steps):
            if store and t % self.K == 0 and t > 0:
                self._save(self.ckpt[t // self.K])
            self.sim.step(1)
            if self._in_window(t + 1):
                self._check(self.lib.lbm_loss(self.h, None, self.kind, _vp(self.weight), self.tw, ctypes.byref(out)))
                loss += out.value
        if store:
            self._save(self.final_state)
        self.sim.synchronize()
        return loss

    # ------------------------------------------------------------ adjoint
    def _adjoint_step(self, state, t, collide):
        """lam <- dL/df^t from lam_next = dL/df^{t+1}, then swap the two."""
        kind = self.kind if self._in_window(t) else N.LOSS_NONE
        fn = self.lib.lbm_adjoint_step_f32 if self.adjoint == "f32" else self.lib.lbm_adjoint_step
        self._check(fn(self.h, _vp(state), _vp(self._lam_next) if collide else None,
                       _vp(self._lam if collide else self._lam_next), collide, kind, _vp(self.weight), self.tw,
                       _vp(self._gF), _vp(self._gS)))
        if collide:
            self._lam, self._lam_next = self._lam_next, self._lam

    def _reverse(self, a, b, level, buf):
        """Adjoint from lam^b (in lam_next) to lam^a over the steps [a, b),
        with f^a in buf."""
        if level == len(self.strides):
            states = [buf] + self._pool(level, b - a - 1)
            if b - a > 1:
                self._load(buf)
                for i in range(1, b - a):
                    self.sim.step(1)
                    self._save(states[i])
            for t in range(b - 1, a - 1, -1):
                self._adjoint_step(states[t - a], t, 1)
            return
        S = self.strides[level]
        starts = list(range(a, b, S))
        subs = [buf] + self._pool(level, len(starts) - 1)
        if len(starts) > 1:
            self._load(buf)
            for i in range(1, len(starts)):
                self.sim.step(S)
                self._save(subs[i])
        for i in reversed(range(len(starts))):
            self._reverse(starts[i], min(b, starts[i] + S), level + 1, subs[i])

    def run_backward(self, grad_force=True):
        """(grad_force (3, plane) or None, grad_porosity (plane,)) after
        run_forward(store=True)."""
        Q, P = self.Q, self.plane
        ldt = torch.float32 if self.adjoint == "f32" else torch.float64
        self._lam_next = torch.zeros((Q, P), dtype=ldt, device=self.dev)
        self._lam = torch.zeros_like(self._lam_next)
        self._gF = torch.zeros((3, P), dtype=torch.float64, device=self.dev) if grad_force else None
        self._gS = torch.zeros((P,), dtype=torch.float64, device=self.dev)
        self._torch_done()
        T = self.steps
        # seed: the final state's loss term (its direct force dependence
        # included); its buffer then serves the finest level's recomputation
        self._adjoint_step(self.final_state, T, 0)
        finest = self._pools.setdefault(len(self.strides), [])
        if not any(b is self.final_state for b in finest):
            finest.insert(0, self.final_state)
        for k in reversed(range(len(self.ckpt))):
            self._reverse(k * self.K, min(T, (k + 1) * self.K), 1, self.ckpt[k])
        self.sim.synchronize()
        gF, gS = self._gF, self._gS
        self._lam = self._lam_next = self._gF = self._gS = None
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
                storage="f64", force=(0.0, 0.0, 0.0), u0=None, device=0, adjoint="f64", arithmetic=None):
    if arithmetic is None:
        arithmetic = "f64" if storage == "f64" else "auto"
    sim = Simulation(nx, ny, nz, lattice=lattice, pattern="ab_push", omega=1.0 / tau, force=force, periodic=periodic,
                     storage=storage, arithmetic=arithmetic, device=device)
    sim.set_solid(solid)
    sim.init_equilibrium(None, u0)
    return Rollout(sim, steps, checkpoint_every, loss, weight, window, adjoint=adjoint)
