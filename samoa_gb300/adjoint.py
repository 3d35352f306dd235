"""Gradient of a gauge-misfit objective through many SWE steps on the GPU.

J(h0, b) = sum_t sum_g (h_{t+1}[gauge g] - obs[t, g])^2 over T steps of the
f-wave step with a frozen dt sequence, as a function of the initial surface
h0 (momentum starts at rest) and the bathymetry b. The reverse sweep calls the
hand-written discrete adjoint of the step (swe_adjoint_step) once per step;
states are recomputed from checkpoints with binomial checkpointing (the
offline schedule of Griewank and Walther's "revolve": with s snapshot slots a
sweep over T steps recomputes every step at most r times, where r is the
smallest integer with C(s + r, s) >= T), so thousands of steps fit in a few
snapshots. Device memory comes from torch; the step and its adjoint are the
C ABI of libsamoa_swe.so.
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _lib
from .swe import SweContext


def _vp(t):
    return C.c_void_p(t.data_ptr())


def binomial_split(length, free):
    """First checkpoint offset for reversing `length` steps when the start state
    is held and `free` more slots are available (revolve's offline rule). With
    c = free + 1 checkpoints and r repetitions, C(c + r, c) steps can be
    reversed; the tail [m, length) gets as many steps as c - 1 checkpoints can
    reverse with r repetitions, the head the rest (Pascal's rule)."""
    if length <= 1 or free <= 0:
        return 1
    c = free + 1
    r = 0
    while math.comb(c + r, c) < length:
        r += 1
    tail = math.comb(c - 1 + r, c - 1)
    return max(1, length - min(tail, length - 1))


def revolve(n_steps, snapshots, ops):
    """Reverse n_steps steps with binomial checkpointing.

    ops provides store(step) -> slot (snapshot of the current state, which is at
    `step`), restore(slot, step), advance(k) (k forward steps), adjoint(t) (the
    reverse of step t, called with the state at step t; it may move the state)
    and release(slot). The state must be at step 0 on entry. adjoint(t) is
    called for t = n_steps - 1 down to 0; at most `snapshots` slots are live.
    """
    def rev(a, b, s, slot_a):
        length = b - a
        if length == 1:
            ops.restore(slot_a, a)
            ops.adjoint(a)
            return
        if s == 0:
            for t in range(b - 1, a - 1, -1):
                ops.restore(slot_a, a)
                ops.advance(t - a)
                ops.adjoint(t)
            return
        m = a + binomial_split(length, s)
        ops.restore(slot_a, a)
        ops.advance(m - a)
        slot_m = ops.store(m)
        rev(m, b, s - 1, slot_m)
        ops.release(slot_m)
        rev(a, m, s, slot_a)

    if n_steps <= 0:
        return
    slot0 = ops.store(0)
    rev(0, n_steps, snapshots - 1, slot0)
    ops.release(slot0)


class GaugeProblem:
    """A frozen mesh, solver parameters, gauges, observations and dt sequence.

    All device work (the C-ABI calls and the torch operations on the cotangents)
    runs on one CUDA stream, so it is ordered without host synchronisation.
    """

    def __init__(self, mesh, params, gauges, obs, dts, snapshots=64, device=0):
        self.mesh = mesh
        self.params = params
        self.n = mesh.n_cells
        self.stride = (self.n + 1) & ~1  # the context's padded cell count
        self.dev = torch.device("cuda", device)
        self.stream = torch.cuda.Stream(device=self.dev)
        with torch.cuda.stream(self.stream):
            self.gauges = torch.as_tensor(np.asarray(gauges, np.int64), device=self.dev)
            self.obs = torch.as_tensor(np.asarray(obs, np.float64), device=self.dev)
        self.dts = np.ascontiguousarray(dts, np.float64)
        self.T = len(self.dts)
        self.snapshots = int(snapshots)
        if self.snapshots < 1:
            raise ValueError("need at least one snapshot slot")
        self.ctx = SweContext(device)
        self.ctx.set_stream(self.stream.cuda_stream)
        self.ctx.set_params(params)
        self.ctx.upload_mesh(mesh)
        with torch.cuda.stream(self.stream):
            self.slots = torch.empty((self.snapshots, 3, self.n), dtype=torch.float64, device=self.dev)
            self.branches = torch.empty((self.T, self.stride), dtype=torch.uint8, device=self.dev)
        self.free = []
        self.stats = {"forward_steps": 0, "adjoint_steps": 0}

    def close(self):
        self.stream.synchronize()
        self.ctx.close()

    # ---- primitives
    def _set_initial(self, h0, b):
        h0 = torch.as_tensor(h0, dtype=torch.float64).detach().cpu().numpy()
        b = torch.as_tensor(b, dtype=torch.float64).detach().cpu().numpy()
        z = np.zeros(self.n)
        self.ctx.upload_mesh(self.mesh)  # resets the step count (traversal parity) to 0
        self.ctx.set_params(self.params)
        self.ctx.upload_state(h0, z, z, b)
        self.ctx.set_time(0.0, float(self.dts[0]) if self.T else 0.0)
        self.ctx.set_dt_sequence(self.dts)

    def _store(self, step):
        slot = self.free.pop()
        s = self.slots[slot]
        got = C.c_int64()
        _lib.check(self.ctx.L.swe_snapshot_store(self.ctx.ptr, _vp(s[0]), _vp(s[1]), _vp(s[2]), C.byref(got)))
        assert got.value == step, (got.value, step)
        return slot

    def _restore(self, slot, step):
        s = self.slots[slot]
        _lib.check(self.ctx.L.swe_snapshot_restore(self.ctx.ptr, _vp(s[0]), _vp(s[1]), _vp(s[2]), step))
        self.cur = step

    def _forward(self, k):
        """k forward steps from self.cur, recording branches and (first time) gauges."""
        L = self.ctx.L
        for _ in range(k):
            t = self.cur
            _lib.check(L.swe_traverse_branches(self.ctx.ptr, 1, _vp(self.branches[t]), self.stride))
            if not self.done[t]:
                _lib.check(L.swe_sample_gauges(self.ctx.ptr, len(self.gauges), _vp(self.gauges), _vp(self.gv[t])))
                self.done[t] = True
            self.cur = t + 1
            self.stats["forward_steps"] += 1

    # ---- objective
    def objective(self, h0, b, record=True):
        """J and the gauge series h_{t+1}[g] of a forward run."""
        self._set_initial(h0, b)
        L = self.ctx.L
        with torch.cuda.stream(self.stream):
            gv = torch.empty((self.T, len(self.gauges)), dtype=torch.float64, device=self.dev)
            _lib.check(L.swe_traverse_gauges(self.ctx.ptr, self.T, len(self.gauges), _vp(self.gauges), _vp(gv)))
            J = float(((gv - self.obs) ** 2).sum().item())
        self.stats["forward_steps"] += self.T
        if record:
            self.gauge_values = gv
        return J

    def gradient(self, h0, b):
        """(J, dJ/dh0, dJ/db) from one checkpointed sweep run inside the library
        (swe_gauge_gradient: the same schedule as gradient_python, no host round
        trips between steps)."""
        self._set_initial(h0, b)
        L = self.ctx.L
        with torch.cuda.stream(self.stream):
            self.gv = torch.empty((self.T, len(self.gauges)), dtype=torch.float64, device=self.dev)
            gh = torch.empty(self.n, dtype=torch.float64, device=self.dev)
            gb = torch.empty(self.n, dtype=torch.float64, device=self.dev)
        self.stream.synchronize()
        J = C.c_double()
        fwd = C.c_int64()
        _lib.check(L.swe_gauge_gradient(self.ctx.ptr, self.T, self.dts.ctypes.data_as(C.c_void_p), self.snapshots,
                                        len(self.gauges), _vp(self.gauges), _vp(self.obs), _vp(self.gv), _vp(gh),
                                        None, None, _vp(gb), C.byref(J), C.byref(fwd)))
        self.stats["forward_steps"] += fwd.value
        self.stats["adjoint_steps"] += self.T
        self.gauge_values = self.gv
        return J.value, gh, gb

    def gradient_python(self, h0, b):
        """(J, dJ/dh0, dJ/db) from one checkpointed sweep driven from Python step
        by step: the first forward descent of the schedule records the gauges
        (for J and its residuals) and every forward step records its branches
        for the reverse step."""
        n = self.n
        L = self.ctx.L
        problem = self
        with torch.cuda.stream(self.stream):
            self.gv = torch.empty((self.T, len(self.gauges)), dtype=torch.float64, device=self.dev)
            self.done = [False] * self.T
            lam = torch.zeros((3, n), dtype=torch.float64, device=self.dev)
            out = torch.zeros_like(lam)
            bbar = torch.zeros(n, dtype=torch.float64, device=self.dev)
            state = {"lam": lam, "out": out}

            class Ops:
                def store(self, step):
                    return problem._store(step)

                def restore(self, slot, step):
                    problem._restore(slot, step)

                def advance(self, k):
                    problem._forward(k)

                def adjoint(self, t):
                    assert problem.cur == t
                    if not problem.done[t]:  # first visit of step t: run it, then step back to x_t
                        problem._forward(1)
                        _lib.check(L.swe_step_back(problem.ctx.ptr))
                        problem.cur = t
                    lam_, out_ = state["lam"], state["out"]
                    lam_[0].index_add_(0, problem.gauges, 2.0 * (problem.gv[t] - problem.obs[t]))
                    _lib.check(L.swe_adjoint_step(problem.ctx.ptr, _vp(problem.branches[t]), _vp(lam_[0]),
                                                  _vp(lam_[1]), _vp(lam_[2]), _vp(out_[0]), _vp(out_[1]),
                                                  _vp(out_[2]), _vp(bbar)))
                    state["lam"], state["out"] = out_, lam_
                    problem.stats["adjoint_steps"] += 1

                def release(self, slot):
                    problem.free.append(slot)

            self._set_initial(h0, b)
            self.cur = 0
            self.free = list(range(self.snapshots))
            revolve(self.T, self.snapshots, Ops())
            J = float(((self.gv - self.obs) ** 2).sum().item())
            gh = state["lam"][0].clone()
        self.stream.synchronize()
        self.gauge_values = self.gv
        return J, gh, bbar


def time_steps(problem, h0, b, k=50):
    """Seconds per forward step and per reverse step (the adjoint kernel with
    recorded branches), on the problem's mesh, from the state (h0, b)."""
    P = problem
    L = P.ctx.L
    P._set_initial(h0, b)
    with torch.cuda.stream(P.stream):
        lam = torch.zeros((3, P.n), dtype=torch.float64, device=P.dev)
        out = torch.zeros_like(lam)
        bbar = torch.zeros(P.n, dtype=torch.float64, device=P.dev)
        P.free = list(range(P.snapshots))
        P.cur = 0
        P.done = [True] * P.T
        slot = P._store(0)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        _lib.check(L.swe_traverse_branches(P.ctx.ptr, 1, _vp(P.branches[0]), P.stride))  # warm-up
        P._restore(slot, 0)
        e0.record(P.stream)
        for _ in range(k):
            _lib.check(L.swe_traverse_branches(P.ctx.ptr, 1, _vp(P.branches[0]), P.stride))
        e1.record(P.stream)
        P._restore(slot, 0)
        for _ in range(k):
            _lib.check(L.swe_adjoint_step(P.ctx.ptr, _vp(P.branches[0]), _vp(lam[0]), _vp(lam[1]), _vp(lam[2]),
                                          _vp(out[0]), _vp(out[1]), _vp(out[2]), _vp(bbar)))
        e2.record(P.stream)
        e2.synchronize()
        P.free.append(slot)
    return e0.elapsed_time(e1) * 1e-3 / k, e1.elapsed_time(e2) * 1e-3 / k


class GaugeMisfit(torch.autograd.Function):
    """J(h0, b) for a GaugeProblem, differentiable with respect to h0 and b."""

    @staticmethod
    def forward(ctx, h0, b, problem):
        J, gh, gb = problem.gradient(h0, b)
        ctx.save_for_backward(gh, gb)
        return torch.tensor(J, dtype=torch.float64, device=h0.device)

    @staticmethod
    def backward(ctx, gJ):
        gh, gb = ctx.saved_tensors
        return gJ * gh.to(gJ.device), gJ * gb.to(gJ.device), None


def record_dts(mesh, params, h0, b, steps, device=0):
    """The CFL dt sequence of an unfrozen forward run from (h0, b), to be frozen."""
    ctx = SweContext(device)
    try:
        ctx.set_params(params)
        ctx.upload_mesh(mesh)
        z = np.zeros(mesh.n_cells)
        ctx.upload_state(np.asarray(h0, np.float64), z, z, np.asarray(b, np.float64))
        from .swe import initial_dt
        ctx.set_time(0.0, initial_dt(mesh, np.asarray(h0), z, z, np.asarray(b), params.courant))
        dts = []
        for _ in range(steps):
            _, dt, _ = ctx.get_time()
            if params.max_time > 0.0:
                dt = min(params.max_time, dt)
            if params.output_time_step > 0.0:
                dt = min(params.output_time_step, dt)
            dts.append(dt)
            ctx.traverse(1)
        ctx.synchronize()
        return np.array(dts)
    finally:
        ctx.close()
