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

    def retarget(self, mesh, gauges, obs, dts):
        """The same problem object on another mesh (and gauges, observations, dt
        sequence): the context's buffers and the snapshot and branch buffers are
        reused where they fit (a windowed run moves through many meshes)."""
        self.stream.synchronize()
        self.mesh = mesh
        self.n = mesh.n_cells
        self.stride = (self.n + 1) & ~1
        self.dts = np.ascontiguousarray(dts, np.float64)
        self.T = len(self.dts)
        with torch.cuda.stream(self.stream):
            self.gauges = torch.as_tensor(np.asarray(gauges, np.int64), device=self.dev)
            self.obs = torch.as_tensor(np.asarray(obs, np.float64), device=self.dev)
            if self.slots.shape[2] < self.n:
                self.slots = torch.empty((self.snapshots, 3, self.n), dtype=torch.float64, device=self.dev)
            if self.branches.shape[0] < self.T or self.branches.shape[1] < self.stride:
                self.branches = torch.empty((max(self.T, self.branches.shape[0]), self.stride), dtype=torch.uint8,
                                            device=self.dev)
        # the mesh goes to the device with the next initial state (_set_initial)

    # ---- primitives
    def _set_initial(self, h0, b, hu0=None, hv0=None):
        h0 = torch.as_tensor(h0, dtype=torch.float64).detach().cpu().numpy()
        b = torch.as_tensor(b, dtype=torch.float64).detach().cpu().numpy()
        z = np.zeros(self.n)
        hu0 = z if hu0 is None else torch.as_tensor(hu0, dtype=torch.float64).detach().cpu().numpy()
        hv0 = z if hv0 is None else torch.as_tensor(hv0, dtype=torch.float64).detach().cpu().numpy()
        self.ctx.upload_mesh(self.mesh)  # resets the step count (traversal parity) to 0
        self.ctx.set_params(self.params)
        self.ctx.upload_state(h0, hu0, hv0, b)
        self.ctx.set_time(0.0, float(self.dts[0]) if self.T else 0.0)
        self.ctx.set_dt_sequence(self.dts)

    def _store(self, step):
        slot = self.free.pop()
        s = self.slots[slot][:, :self.n]
        got = C.c_int64()
        _lib.check(self.ctx.L.swe_snapshot_store(self.ctx.ptr, _vp(s[0]), _vp(s[1]), _vp(s[2]), C.byref(got)))
        assert got.value == step, (got.value, step)
        return slot

    def _restore(self, slot, step):
        s = self.slots[slot][:, :self.n]
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
    def objective(self, h0, b, record=True, hu0=None, hv0=None):
        """J and the gauge series h_{t+1}[g] of a forward run (initial momenta
        hu0, hv0; at rest by default)."""
        self._set_initial(h0, b, hu0, hv0)
        L = self.ctx.L
        with torch.cuda.stream(self.stream):
            gv = torch.empty((self.T, len(self.gauges)), dtype=torch.float64, device=self.dev)
            _lib.check(L.swe_traverse_gauges(self.ctx.ptr, self.T, len(self.gauges), _vp(self.gauges), _vp(gv)))
            J = float(((gv - self.obs) ** 2).sum().item())
        self.stats["forward_steps"] += self.T
        if record:
            self.gauge_values = gv
        return J

    def objective_frozen(self, h0, b, record):
        """J of a branch-frozen forward run (swe_traverse_frozen, the f-wave):
        record=True runs from (h0, b) recording every edge's and cell's branch
        decisions; record=False runs again taking every decision from the last
        recording, so J is smooth near the recorded run and its finite
        differences check the discrete adjoint without crossing a kink."""
        self._set_initial(h0, b)
        L = self.ctx.L
        counts = self.ctx.task_counts()
        es = counts["tasks"] + counts["cross_edges"]
        with torch.cuda.stream(self.stream):
            if record or getattr(self, "frozen", None) is None:
                self.frozen = (torch.empty((self.T, self.stride), dtype=torch.uint8, device=self.dev),
                               torch.empty((self.T, es), dtype=torch.int16, device=self.dev))
            br, ed = self.frozen
            if ed.shape[1] != es:
                raise ValueError("the recording belongs to another mesh")
            gv = torch.empty((self.T, len(self.gauges)), dtype=torch.float64, device=self.dev)
            _lib.check(L.swe_traverse_frozen(self.ctx.ptr, self.T, 1 if record else 2, _vp(br), self.stride, _vp(ed),
                                             es, len(self.gauges), _vp(self.gauges), _vp(gv)))
            J = float(((gv - self.obs) ** 2).sum().item())
        self.stats["forward_steps"] += self.T
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

    def gradient_python(self, h0, b, hu0=None, hv0=None, lam_end=None, full=False):
        """(J, dJ/dh0, dJ/db) from one checkpointed sweep driven from Python step
        by step: the first forward descent of the schedule records the gauges
        (for J and its residuals) and every forward step records its branches
        for the reverse step. The initial momenta (hu0, hv0) default to rest;
        lam_end (3 x n, optional) is the cotangent of the final state, for a
        window of a longer run. With full, the gradient in h0 is the whole
        initial-state cotangent (3 x n)."""
        n = self.n
        L = self.ctx.L
        problem = self
        with torch.cuda.stream(self.stream):
            self.gv = torch.empty((self.T, len(self.gauges)), dtype=torch.float64, device=self.dev)
            self.done = [False] * self.T
            lam = torch.zeros((3, n), dtype=torch.float64, device=self.dev)
            if lam_end is not None:
                lam.copy_(torch.as_tensor(lam_end, dtype=torch.float64, device=self.dev))
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

            self._set_initial(h0, b, hu0, hv0)
            self.cur = 0
            self.free = list(range(self.snapshots))
            revolve(self.T, self.snapshots, Ops())
            J = float(((self.gv - self.obs) ** 2).sum().item())
            gh = state["lam"].clone() if full else state["lam"][0].clone()
        self.stream.synchronize()
        self.gauge_values = self.gv
        return J, gh, bbar


def time_steps(problem, h0, b, k=50):
    """Seconds per forward step and per reverse step (the adjoint kernel with
    recorded branches), on the problem's mesh, from the state (h0, b). The
    reverse steps take seeded random cotangents on every cell (a zero
    cotangent lets the kernel skip an edge, which would not time the reverse)."""
    P = problem
    L = P.ctx.L
    P._set_initial(h0, b)
    with torch.cuda.stream(P.stream):
        gen = torch.Generator(device=P.dev)
        gen.manual_seed(0)
        lam = torch.randn((3, P.n), dtype=torch.float64, device=P.dev, generator=gen)
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


def locate_points(vertices, points):
    """Index of the cell containing each point (unit-square coordinates; the
    first cell in traversal order for a point on an edge): float64[n, 3, 2]
    vertices, float64[g, 2] points -> int64[g]."""
    v = np.asarray(vertices, np.float64)
    a, b, c = v[:, 0], v[:, 1], v[:, 2]
    out = np.empty(len(points), np.int64)
    for i, (x, y) in enumerate(np.asarray(points, np.float64)):
        def side(p, q):
            return (q[:, 0] - p[:, 0]) * (y - p[:, 1]) - (q[:, 1] - p[:, 1]) * (x - p[:, 0])
        s0, s1, s2 = side(a, b), side(b, c), side(c, a)
        tol = 1e-15
        inside = ((s0 >= -tol) & (s1 >= -tol) & (s2 >= -tol)) | ((s0 <= tol) & (s1 <= tol) & (s2 <= tol))
        hit = np.flatnonzero(inside)
        if len(hit) == 0:
            raise ValueError("point (%g, %g) lies outside the mesh" % (x, y))
        out[i] = hit[0]
    return out


class Transfer:
    """The order-0 state transfer of one remesh (src/Samoa/Tools_lagrange_basis.f90:139-220):
    a new cell copies its source cell (kept or refined) or averages two merged
    siblings, 0.5 * (q[s] + q[s + 1]); and its adjoint."""

    def __init__(self, old_depth, new_depth, src):
        self.src = np.asarray(src, np.int64)
        self.merged = np.asarray(new_depth, np.int64) < np.asarray(old_depth, np.int64)[self.src]
        self.n_old = len(old_depth)

    def apply(self, q):
        q = np.asarray(q, np.float64)
        out = q[self.src].copy()
        m = self.merged
        out[m] = 0.5 * (q[self.src[m]] + q[self.src[m] + 1])
        return out

    def adjoint(self, qbar):
        qbar = np.asarray(qbar, np.float64)
        out = np.zeros(self.n_old)
        k = ~self.merged
        np.add.at(out, self.src[k], qbar[k])
        m = self.merged
        np.add.at(out, self.src[m], 0.5 * qbar[m])
        np.add.at(out, self.src[m] + 1, 0.5 * qbar[m])
        return out


class WindowedGaugeProblem:
    """J over consecutive windows of `window` steps, each on a frozen mesh: after
    a window the mesh is adapted from its last step's refinement flags
    (swe_mesh_adapt: conformity closure, refine/coarsen), the state and the
    bathymetry carried over by the order-0 transfer, and the gauge points
    located on the new mesh. The first evaluation fixes the mesh sequence and
    the transfers; later evaluations (objective, gradient, finite differences)
    replay them, so J is a function of (h0, b) on the first mesh with the
    adaptive meshes frozen per window. The gradient chains the windows'
    checkpointed adjoints (GaugeProblem.gradient_python with the next window's
    initial cotangent pulled back through the transfer as the final cotangent).

    gauge_points: float64[G, 2] in world coordinates; obs: float64[T, G]; dts: the
    frozen dt of each of the T steps."""

    def __init__(self, mesh0, cfg, gauge_points, obs, dts, window=50, snapshots=64, device=0):
        from .swe import mesh_from_depths
        if mesh0.vertices is None:
            mesh0 = mesh_from_depths(mesh0.depth, centroids=True, vertices=True)
        self.mesh0 = mesh0
        self.cfg = cfg
        self.params = cfg.params()
        pts = np.asarray(gauge_points, np.float64)
        self.points_unit = (pts - np.asarray(cfg.offset, np.float64)) / cfg.scaling
        self.obs = np.asarray(obs, np.float64)
        self.dts = np.asarray(dts, np.float64)
        self.T = len(self.dts)
        self.window = int(window)
        self.snapshots = int(snapshots)
        self.device = device
        self.plan = None
        self.stats = {"windows": 0, "cells": []}

    def _windows(self):
        return [(k, min(k + self.window, self.T)) for k in range(0, self.T, self.window)]

    def _forward(self, h0, b0, record_plan, frozen=None):
        """Run all windows from (h0, b0) at rest; returns J, the initial states of
        the windows and (first run) the meshes, gauges and transfers. frozen:
        None (plain steps), "record" (branch-frozen runs recording every window's
        decisions) or "replay" (taking them from the last recording)."""
        from .swe import adapt
        if frozen == "record":
            self.frozen = []
        ctx = SweContext(self.device)
        try:
            ctx.set_params(self.params)
            h, hu, hv = (np.asarray(h0, np.float64).copy(), np.zeros(self.mesh0.n_cells),
                         np.zeros(self.mesh0.n_cells))
            b = np.asarray(b0, np.float64).copy()
            starts, J = [], 0.0
            meshes, gauges, transfers = ([], [], []) if record_plan else (None, None, None)
            mesh = self.mesh0
            for w, (t0, t1) in enumerate(self._windows()):
                if not record_plan:
                    mesh = self.plan["meshes"][w]
                gw = locate_points(mesh.vertices, self.points_unit) if record_plan else self.plan["gauges"][w]
                if record_plan:
                    meshes.append(mesh)
                    gauges.append(gw)
                starts.append((h.copy(), hu.copy(), hv.copy(), b.copy()))
                ctx.upload_mesh(mesh)
                ctx.upload_state(h, hu, hv, b)
                ctx.set_time(0.0, float(self.dts[t0]))
                ctx.set_dt_sequence(self.dts[t0:t1])
                dev = torch.device("cuda", self.device)
                gi = torch.as_tensor(gw, dtype=torch.int64, device=dev)
                gv = torch.empty((t1 - t0, len(gw)), dtype=torch.float64, device=dev)
                if frozen is None:
                    _lib.check(ctx.L.swe_traverse_gauges(ctx.ptr, t1 - t0, len(gw), _vp(gi), _vp(gv)))
                else:
                    counts = ctx.task_counts()
                    es = counts["tasks"] + counts["cross_edges"]
                    stride = (mesh.n_cells + 1) & ~1
                    if frozen == "record":
                        self.frozen.append((torch.empty((t1 - t0, stride), dtype=torch.uint8, device=dev),
                                            torch.empty((t1 - t0, es), dtype=torch.int16, device=dev)))
                    br, ed = self.frozen[w]
                    if ed.shape[1] != es:
                        raise ValueError("the recording belongs to another mesh")
                    torch.cuda.synchronize(dev)
                    _lib.check(ctx.L.swe_traverse_frozen(ctx.ptr, t1 - t0, 1 if frozen == "record" else 2, _vp(br),
                                                         stride, _vp(ed), es, len(gw), _vp(gi), _vp(gv)))
                ctx.synchronize()
                J += float(((gv.cpu().numpy() - self.obs[t0:t1]) ** 2).sum())
                h, hu, hv, _ = ctx.download_state()
                if t1 < self.T:
                    if record_plan:
                        flags, _ = ctx.refinements()
                        new, _, src = adapt(mesh, flags, with_source=True)
                        tr = Transfer(mesh.depth, new.depth, src)
                        transfers.append(tr)
                        mesh = new
                    else:
                        tr = self.plan["transfers"][w]
                    h, hu, hv, b = tr.apply(h), tr.apply(hu), tr.apply(hv), tr.apply(b)
            if record_plan:
                self.plan = {"meshes": meshes, "gauges": gauges, "transfers": transfers}
                self.stats["cells"] = [m.n_cells for m in meshes]
            return J, starts
        finally:
            ctx.close()

    def objective(self, h0, b0):
        J, _ = self._forward(h0, b0, self.plan is None)
        return J

    def objective_frozen(self, h0, b0, record):
        """J with the plan's meshes and transfers and, in every window, every
        branch decision of the f-wave step taken from a recorded run
        (swe_traverse_frozen): record=True runs from (h0, b0) and records,
        record=False replays the last recording. Near the recorded run J is then
        smooth, so its finite differences check the adjoint without crossing a
        kink. The plan is fixed first if no run has fixed it."""
        if self.plan is None:
            self._forward(h0, b0, True)
        if not record and getattr(self, "frozen", None) is None:
            raise ValueError("record a branch-frozen run first")
        J, _ = self._forward(h0, b0, False, frozen="record" if record else "replay")
        return J

    def gradient(self, h0, b0):
        """(J, dJ/dh0, dJ/db0) on the first mesh."""
        J, starts = self._forward(h0, b0, self.plan is None)
        wins = self._windows()
        lam_end, bbar_next = None, None
        Jsum = 0.0
        big = max(range(len(wins)), key=lambda w: self.plan["meshes"][w].n_cells)
        P = GaugeProblem(self.plan["meshes"][big], self.params, self.plan["gauges"][big],
                         self.obs[wins[big][0]:wins[big][1]], self.dts[wins[big][0]:wins[big][1]],
                         snapshots=min(self.snapshots, self.window), device=self.device)
        try:
            for w in range(len(wins) - 1, -1, -1):
                t0, t1 = wins[w]
                h, hu, hv, b = starts[w]
                P.retarget(self.plan["meshes"][w], self.plan["gauges"][w], self.obs[t0:t1], self.dts[t0:t1])
                Jw, lam0, bbar = P.gradient_python(h, b, hu, hv, lam_end=lam_end, full=True)
                lam0 = lam0.cpu().numpy()
                bbar = bbar.cpu().numpy()
                Jsum += Jw
                if bbar_next is not None:
                    bbar = bbar + bbar_next
                if w > 0:
                    tr = self.plan["transfers"][w - 1]
                    lam_end = np.stack([tr.adjoint(lam0[q]) for q in range(3)])
                    bbar_next = tr.adjoint(bbar)
                else:
                    gh, gb = lam0[0], bbar
        finally:
            P.close()
        self.stats["windows"] = len(wins)
        # J of the forward run, summed as objective() sums it (window by window on
        # the host); the sweep's own sum of the windows' J takes another order
        self.stats["J_sweep"] = Jsum
        return J, gh, gb


class GaugeMisfit(torch.autograd.Function):
    """J(h0, b) for a GaugeProblem (or a WindowedGaugeProblem), differentiable
    with respect to h0 and b. forward is one forward run (problem.objective);
    backward runs the checkpointed reverse sweep (problem.gradient) from the
    saved inputs, so an evaluation that needs no gradient pays no sweep."""

    @staticmethod
    def forward(ctx, h0, b, problem):
        J = problem.objective(h0, b)
        ctx.problem = problem
        ctx.save_for_backward(h0, b)
        return torch.tensor(J, dtype=torch.float64, device=h0.device)

    @staticmethod
    def backward(ctx, gJ):
        h0, b = ctx.saved_tensors
        _, gh, gb = ctx.problem.gradient(h0, b)
        gh = torch.as_tensor(gh, dtype=torch.float64).to(gJ.device)
        gb = torch.as_tensor(gb, dtype=torch.float64).to(gJ.device)
        return gJ * gh, gJ * gb, None


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
