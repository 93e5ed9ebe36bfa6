"""Host logic of the checkpointed reverse sweep (no GPU): a fake handle whose
"state" is the step count checks that every adjoint step is handed the state
of its own step, for single- and multi-level checkpoint strides."""
import ctypes

import pytest
import torch

from lbmminiapp_gb300 import adjoint as A
from lbmminiapp_gb300 import _native as N


class FakeLib:
    """Stands in for the C ABI: a state buffer holds the step count t as an
    int64 in its first 8 bytes; the handle's current state is sim.t."""

    def __init__(self, sim):
        self.sim = sim
        self.calls = []
        self.copies = 0

    def lbm_copy_state(self, h, vp, to_handle):
        cell = ctypes.c_int64.from_address(vp.value)
        if to_handle:
            self.sim.t = cell.value
        else:
            cell.value = self.sim.t
        self.copies += 1
        return 0

    def lbm_loss(self, h, state, kind, weight, tw, out):
        out._obj.value = float(self.sim.t)
        return 0

    def _adj(self, h, state, lam_next, lam, collide, kind, weight, tw, gF, gS):
        self.calls.append((ctypes.c_int64.from_address(state.value).value, collide, kind))
        return 0

    lbm_adjoint_step = _adj
    lbm_adjoint_step_f32 = _adj

    def lbm_set_fields_device(self, *a):
        return 0


class FakeSim:
    pattern = "ab_push"
    Q = 19
    shape = (2, 2, 2)
    ncell = 8

    def __init__(self):
        self.t = 0
        self.steps_run = 0
        self.lib = FakeLib(self)
        self.h = object()

        class Info:
            plane_stride = 8
            buffer_bytes = 64
        self.info = Info()

        class Cfg:
            device = 0
        self.cfg = Cfg()

    def step(self, n=1):
        self.t += n
        self.steps_run += n

    def synchronize(self):
        pass


@pytest.mark.parametrize("steps,strides", [(24, 8), (24, (8, 3)), (25, (9, 4, 2)), (7, 10), (30, (10, 1)),
                                           (2000, (729, 243, 81, 27, 9, 3)), (2000, (100, 10))])
def test_reverse_sweep_sees_each_state(steps, strides):
    sim = FakeSim()
    w = torch.zeros(3, 8, dtype=torch.float64)
    r = A.Rollout(sim, steps, strides, "velocity", w, (steps - 2, steps), device="cpu")
    loss = r.run_forward(store=True)
    assert loss == sum(range(steps - 2, steps + 1))
    forward_steps = sim.steps_run
    sim.lib.calls.clear()
    r.run_backward(grad_force=False)
    calls = sim.lib.calls
    # the seed reads the final state, then one collide step per time step, last to first
    assert calls[0] == (steps, 0, N.LOSS_VELOCITY)
    assert [c[0] for c in calls[1:]] == list(range(steps - 1, -1, -1))
    assert all(c[1] == 1 for c in calls[1:])
    assert [c[2] == N.LOSS_VELOCITY for c in calls[1:]] == [steps - 2 <= t <= steps for t in range(steps - 1, -1, -1)]
    # recomputation: at most one forward pass per checkpoint level
    levels = 1 if isinstance(strides, int) else len(strides)
    assert sim.steps_run - forward_steps <= levels * steps
    # buffers held: the checkpoints, the pools and the final state's buffer
    held = len(r.ckpt) + sum(len(p) for p in r._pools.values())
    assert held <= A.checkpoint_buffers(steps, strides)


def test_strides_must_decrease():
    sim = FakeSim()
    w = torch.zeros(3, 8, dtype=torch.float64)
    for bad in [(8, 8), (3, 8), (8, 0), ()]:
        with pytest.raises(ValueError):
            A.Rollout(sim, 24, bad, "velocity", w, (20, 24), device="cpu")
    with pytest.raises(ValueError):
        A.Rollout(sim, 24, 8, "velocity", w, (20, 24), adjoint="f16", device="cpu")


def test_checkpoint_buffer_counts():
    assert A.checkpoint_buffers(2000, 100) == 20 + 99
    assert A.checkpoint_buffers(2000, (100, 10)) == 20 + 9 + 9
    assert A.checkpoint_buffers(2000, (729, 243, 81, 27, 9, 3)) == 3 + 5 * 2 + 2
