"""Host-side mirror of sam(oa)^2's SWE Euler time-step traversal over the C ABI.

The reference calls ``swe%euler%traverse(grid)`` once per time step
(src/SWE/SWE.f90:393). Here a :class:`Grid` holds the Sierpinski mesh and the
cell state ``Q = (h, hu, hv, b)`` (h is the surface elevation, depth = h - b,
src/SWE/SWE_data_types.f90:42-65) plus ``r_time``, ``r_dt`` and ``r_dt_new``;
:class:`SweEulerTimestepTraversal` runs the step on the GPU through
libsamoa_swe.so and leaves the grid updated, with refinement flags and
``i_refinements_issued`` like the reference traversal.
"""
import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib

FWAVE, AUG_RIEMANN, LF, LF_BATH, LLF, LLF_BATH = 1, 3, 10, 11, 12, 13
SOLVERS = {"fwave": FWAVE, "aug_riemann": AUG_RIEMANN, "lf": LF, "lfbath": LF_BATH, "llf": LLF,
           "llfbath": LLF_BATH}
BC_OUTFLOW, BC_SLIP, BC_NOSLIP = 0, 1, 2
BOUNDARIES = {"outflow": BC_OUTFLOW, "slip": BC_SLIP, "noslip": BC_NOSLIP}

G = 9.80665  # src/SWE/SWE_data_types.f90:34


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


@dataclass
class Config:
    """The cfg fields the step reads (src/Config.f90:30-121; SWE defaults of :183)."""
    flux_solver: str = "fwave"
    boundary: str = "outflow"
    courant_number: float = 0.45
    dry_tolerance: float = 0.01
    scaling: float = 1.0
    offset: tuple = (0.0, 0.0)
    i_min_depth: int = 0
    i_max_depth: int = 14
    r_max_time: float = -1.0
    r_output_time_step: float = -1.0

    def params(self):
        return _lib.SweParams(SOLVERS[self.flux_solver], BOUNDARIES[self.boundary], self.dry_tolerance,
                              self.courant_number, self.scaling, self.i_min_depth, self.i_max_depth,
                              self.r_max_time, self.r_output_time_step)


@dataclass
class Mesh:
    """Cells in traversal order and their edge streams (the C-ABI layout)."""
    depth: np.ndarray          # int8[n]
    plotter: np.ndarray        # int8[n]
    edge_cells: np.ndarray     # int64[ne, 2]
    edge_local: np.ndarray     # int8[ne, 2], 1..3
    bnd_cell: np.ndarray       # int64[nb]
    bnd_local: np.ndarray      # int8[nb]
    centroids: np.ndarray = None  # float64[n, 2] in the unit square (optional)
    version: int = 0
    vertices: np.ndarray = None   # float64[n, 3, 2] in the unit square (optional)

    @property
    def n_cells(self):
        return len(self.depth)


def uniform_mesh(depth, centroids=True):
    """Uniform Sierpinski mesh of the unit square at reference depth ``depth`` (2^(depth+1) cells)."""
    L = _lib.load()
    n, ne, nb = C.c_int64(), C.c_int64(), C.c_int64()
    _lib.check(L.swe_mesh_uniform(depth, C.byref(n), C.byref(ne), C.byref(nb), *([None] * 8)))
    n, ne, nb = n.value, ne.value, nb.value
    d = np.empty(n, np.int8)
    p = np.empty(n, np.int8)
    ec = np.empty((ne, 2), np.int64)
    el = np.empty((ne, 2), np.int8)
    bc = np.empty(nb, np.int64)
    bl = np.empty(nb, np.int8)
    cen = np.empty((n, 2), np.float64) if centroids else None
    _lib.check(L.swe_mesh_uniform(depth, None, None, None, _p(d), _p(p), _p(ec), _p(el), _p(bc), _p(bl), _p(cen)))
    return Mesh(d, p, ec, el, bc, bl, cen)


def mesh_from_depths(depths, centroids=True, vertices=False):
    """Mesh of the conforming Sierpinski tree whose leaves, in traversal order,
    have the given depths (swe_mesh_build)."""
    L = _lib.load()
    d = np.ascontiguousarray(depths, np.int8)
    n = len(d)
    # 2 * n_edges + n_bnd = 3 * n: arrays of that bound take one walk (the
    # untouched tails are never paged in)
    ne, nb = C.c_int64(), C.c_int64()
    p = np.empty(n, np.int8)
    ec = np.empty(((3 * n) // 2, 2), np.int64)
    el = np.empty(((3 * n) // 2, 2), np.int8)
    bc = np.empty(3 * n, np.int64)
    bl = np.empty(3 * n, np.int8)
    cen = np.empty((n, 2), np.float64) if centroids else None
    ver = np.empty((n, 3, 2), np.float64) if vertices else None
    _lib.check(L.swe_mesh_build(n, _p(d), C.byref(ne), C.byref(nb), _p(p), _p(ec), _p(el), _p(bc), _p(bl), _p(cen),
                                _p(ver)))
    ne, nb = ne.value, nb.value
    return Mesh(d.copy(), p, ec[:ne], el[:ne], bc[:nb].copy(), bl[:nb].copy(), cen, vertices=ver)


def adapt(mesh, flags, h=None, hu=None, hv=None, b=None, with_source=False):
    """One remesh from refinement flags (-1, 0, 1; the step's output): returns the
    new mesh and the transferred (h, hu, hv, b) (None where not given), and with
    with_source also each new cell's source cell."""
    L = _lib.load()
    f = np.ascontiguousarray(flags, np.int8)
    ins = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (h, hu, hv, b)]
    n_out = C.c_int64()
    cap = 2 * mesh.n_cells + 64  # enough unless most cells refine twice; else a second call with the count
    for _ in range(2):
        d = np.empty(cap, np.int8)
        src = np.empty(cap, np.int64)
        outs = [None if a is None else np.empty(cap, np.float64) for a in ins]
        rc = L.swe_mesh_adapt(mesh.n_cells, _p(mesh.depth), _p(f), *[_p(a) for a in ins], cap, C.byref(n_out),
                              _p(d), _p(src), *[_p(a) for a in outs])
        if rc == 0 or n_out.value <= cap:
            _lib.check(rc)
            break
        cap = n_out.value
    m = n_out.value
    d, src = d[:m], src[:m]
    outs = [None if a is None else a[:m] for a in outs]
    new = mesh_from_depths(d, centroids=mesh.centroids is not None, vertices=mesh.vertices is not None)
    return (new, outs, src) if with_source else (new, outs)


@dataclass
class Grid:
    """A mesh plus the SWE cell state and the time-stepping scalars of t_grid."""
    mesh: Mesh
    h: np.ndarray
    hu: np.ndarray
    hv: np.ndarray
    b: np.ndarray
    r_time: float = 0.0
    r_dt: float = 0.0
    r_dt_new: float = 0.0
    refinement: np.ndarray = None
    i_refinements_issued: int = 0
    steps_since_upload: int = 0
    _dirty: bool = field(default=True, repr=False)

    def mark_dirty(self):
        """Call after changing the host state arrays so the next traverse uploads them."""
        self._dirty = True


class SweContext:
    """Owner of one swe_ctx (device buffers, stream, device scalars)."""

    def __init__(self, device=0):
        self.L = _lib.load()
        self.ptr = C.c_void_p()
        _lib.check(self.L.swe_create(C.byref(self.ptr), device))
        self.n_cells = 0

    def close(self):
        if self.ptr:
            self.L.swe_destroy(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params):
        _lib.check(self.L.swe_set_params(self.ptr, C.byref(params)))

    def set_stream(self, stream_handle):
        _lib.check(self.L.swe_set_stream(self.ptr, C.c_void_p(stream_handle)))

    def set_tiling(self, segment_cells=0, block_threads=0):
        _lib.check(self.L.swe_set_tiling(self.ptr, segment_cells, block_threads))

    def set_staging(self, depth):
        """Segments staged ahead per CTA: 1 or 2 (swe_set_staging)."""
        _lib.check(self.L.swe_set_staging(self.ptr, int(depth)))

    def set_arith(self, mode):
        """"strict" (bit-exact FP64, default) or "fma" (fused multiply-adds, within a few ulps per step)."""
        _lib.check(self.L.swe_set_arith(self.ptr, {"strict": 0, "fma": 1}[mode]))

    def get_tiling(self):
        a, b = C.c_int32(), C.c_int32()
        _lib.check(self.L.swe_get_tiling(self.ptr, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_cross_pass(self, mode):
        """How edges between two segments are solved: "auto" (default), "pass" (once, by a kernel
        before the step kernel) or "inkernel" (by both segments' CTAs); bit-identical results."""
        _lib.check(self.L.swe_set_cross_pass(self.ptr, {"auto": 0, "pass": 1, "inkernel": 2}[mode]))

    def set_segment_order(self, mode):
        """The order segments are handed out in: "spread" (bit-reversed within each instance,
        mixing wet and dry work on every SM), "curve", or "auto" (default: spread from 2048
        segments on); bit-identical results."""
        _lib.check(self.L.swe_set_segment_order(self.ptr, {"curve": 0, "spread": 1, "auto": 2}[mode]))

    def task_counts(self):
        """Segments, edge tasks, edges between two segments and kernel launches per step
        of the uploaded mesh."""
        s, t, x, k = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int32()
        _lib.check(self.L.swe_get_task_counts(self.ptr, C.byref(s), C.byref(t), C.byref(x), C.byref(k)))
        return {"segments": s.value, "tasks": t.value, "cross_edges": x.value, "launches_per_step": k.value}

    def upload_mesh(self, mesh):
        ec = np.ascontiguousarray(mesh.edge_cells, np.int64)
        el = np.ascontiguousarray(mesh.edge_local, np.int8)
        bc = np.ascontiguousarray(mesh.bnd_cell, np.int64)
        bl = np.ascontiguousarray(mesh.bnd_local, np.int8)
        d = np.ascontiguousarray(mesh.depth, np.int8)
        p = np.ascontiguousarray(mesh.plotter, np.int8)
        _lib.check(self.L.swe_mesh_upload(self.ptr, len(d), _p(d), _p(p), len(ec), _p(ec), _p(el), len(bc), _p(bc),
                                          _p(bl)))
        self.n_cells = len(d)

    def upload_state(self, h, hu, hv, b):
        arrs = [np.ascontiguousarray(x, np.float64) for x in (h, hu, hv, b)]
        for a in arrs:
            if a.shape != (self.n_cells,):
                raise ValueError("state arrays must have shape (%d,)" % self.n_cells)
        _lib.check(self.L.swe_state_upload(self.ptr, *[_p(a) for a in arrs]))

    def download_state(self, out=None):
        if out is None:
            out = [np.empty(self.n_cells, np.float64) for _ in range(4)]
        _lib.check(self.L.swe_state_download(self.ptr, *[_p(a) for a in out]))
        return out

    def device_state(self):
        ptrs = [C.c_void_p() for _ in range(4)]
        _lib.check(self.L.swe_state_device(self.ptr, *[C.byref(q) for q in ptrs]))
        return [q.value for q in ptrs]

    def set_time(self, time, dt):
        _lib.check(self.L.swe_set_time(self.ptr, float(time), float(dt)))

    def get_time(self):
        t, dt, dn = C.c_double(), C.c_double(), C.c_double()
        _lib.check(self.L.swe_get_time(self.ptr, C.byref(t), C.byref(dt), C.byref(dn)))
        return t.value, dt.value, dn.value

    def traverse(self, n_steps=1):
        _lib.check(self.L.swe_traverse(self.ptr, int(n_steps)))

    def step_host(self, h, hu, hv, b, h_out, hu_out, hv_out, flags_out=None):
        """One step reading (h, hu, hv, b) and writing (h_out, hu_out, hv_out,
        flags_out) where they live: torch tensors in pinned host memory or on
        the context's device (b and flags_out may be None). Asynchronous."""
        ptr = lambda t: None if t is None else C.c_void_p(t.data_ptr())
        for t in (h, hu, hv, b, h_out, hu_out, hv_out, flags_out):
            if t is not None and (not t.is_contiguous() or t.numel() < self.n_cells):
                raise ValueError("arrays must be contiguous with n_cells elements")
        _lib.check(self.L.swe_step_host(self.ptr, ptr(h), ptr(hu), ptr(hv), ptr(b), ptr(h_out), ptr(hu_out),
                                        ptr(hv_out), ptr(flags_out)))

    def refinements(self, flags=None):
        if flags is None:
            flags = np.empty(self.n_cells, np.int8)
        n = C.c_int64()
        _lib.check(self.L.swe_get_refinements(self.ptr, _p(flags), C.byref(n)))
        return flags, n.value

    def step_count(self):
        s = C.c_int64()
        _lib.check(self.L.swe_get_step_count(self.ptr, C.byref(s)))
        return s.value

    def synchronize(self):
        _lib.check(self.L.swe_synchronize(self.ptr))

    def traverse_graph(self, n_steps):
        """n_steps steps as one CUDA graph (captured on first use, replayed afterwards)."""
        _lib.check(self.L.swe_traverse_graph(self.ptr, int(n_steps)))

    def set_dt_sequence(self, dts):
        """Freeze the dt of the next len(dts) steps (shape (steps,) or (steps, n_instances)); None clears."""
        if dts is None or len(dts) == 0:
            _lib.check(self.L.swe_set_dt_sequence(self.ptr, 0, None))
            return
        a = np.ascontiguousarray(dts, np.float64)
        _lib.check(self.L.swe_set_dt_sequence(self.ptr, a.shape[0], _p(a)))


class SweEnsemble(SweContext):
    """Many independent SWE instances stepped together: one kernel launch per
    time step for all instances, each with its own parameters and dt."""

    def upload_meshes(self, meshes):
        nc = np.array([m.n_cells for m in meshes], np.int64)
        ne = np.array([len(m.edge_cells) for m in meshes], np.int64)
        nb = np.array([len(m.bnd_cell) for m in meshes], np.int64)
        cat = lambda xs, dt: np.ascontiguousarray(np.concatenate(xs), dt)
        d = cat([m.depth for m in meshes], np.int8)
        p = cat([m.plotter for m in meshes], np.int8)
        ec = cat([m.edge_cells.reshape(-1, 2) for m in meshes], np.int64)
        el = cat([m.edge_local.reshape(-1, 2) for m in meshes], np.int8)
        bc = cat([m.bnd_cell for m in meshes], np.int64)
        bl = cat([m.bnd_local for m in meshes], np.int8)
        _lib.check(self.L.swe_ensemble_mesh_upload(self.ptr, len(meshes), _p(nc), _p(ne), _p(nb), _p(d), _p(p),
                                                   _p(ec), _p(el), _p(bc), _p(bl)))
        self.n_instances = len(meshes)
        self.sizes = nc
        self.n_cells = int(nc.sum())

    def set_params_list(self, params):
        arr = (_lib.SweParams * len(params))(*params)
        _lib.check(self.L.swe_ensemble_set_params(self.ptr, arr))

    def set_times(self, times, dts):
        t = np.ascontiguousarray(times, np.float64)
        d = np.ascontiguousarray(dts, np.float64)
        _lib.check(self.L.swe_ensemble_set_time(self.ptr, _p(t), _p(d)))

    def get_times(self):
        t, d, dn = (np.empty(self.n_instances) for _ in range(3))
        _lib.check(self.L.swe_ensemble_get_time(self.ptr, _p(t), _p(d), _p(dn)))
        return t, d, dn

    def refinements_all(self):
        f = np.empty(self.n_cells, np.int8)
        n = np.empty(self.n_instances, np.int64)
        _lib.check(self.L.swe_ensemble_get_refinements(self.ptr, _p(f), _p(n)))
        return f, n

    def split(self, a):
        return np.split(a, np.cumsum(self.sizes)[:-1])


class SweEulerTimestepTraversal:
    """GPU drop-in for t_swe_euler_timestep_traversal (src/SWE/SWE_euler_timestep.f90).

    ``traverse(grid)`` performs one explicit Euler step exactly like
    ``swe%euler%traverse(grid)``: uses ``grid.r_dt``, advances ``grid.r_time``,
    sets ``grid.r_dt = courant * min(volume / sum(len * speed))``, the
    refinement flags and ``grid.i_refinements_issued``. The mesh is uploaded
    when its ``version`` changes (a remesh), the state when the grid is dirty.
    With ``sync_state=False`` the state stays on the device between calls
    (call :meth:`fetch` to read it back).
    """

    def __init__(self, cfg: Config, device=0):
        self.cfg = cfg
        self.ctx = SweContext(device)
        self.ctx.set_params(cfg.params())
        self._mesh_key = None

    def set_tiling(self, segment_cells=0, block_threads=0, staging_depth=None):
        self.ctx.set_tiling(segment_cells, block_threads)
        if staging_depth:
            self.ctx.set_staging(staging_depth)

    def _ensure(self, grid):
        key = (id(grid.mesh), grid.mesh.version)
        if key != self._mesh_key:
            self.ctx.upload_mesh(grid.mesh)
            self._mesh_key = key
            grid._dirty = True
            grid.steps_since_upload = 0
        if grid._dirty:
            self.ctx.upload_state(grid.h, grid.hu, grid.hv, grid.b)
            self.ctx.set_time(grid.r_time, grid.r_dt)
            grid._dirty = False

    def traverse(self, grid: Grid, steps=1, sync_state=True, flags=True):
        self.ctx.set_params(self.cfg.params())
        self._ensure(grid)
        self.ctx.traverse(steps)
        grid.steps_since_upload += steps
        self.ctx.synchronize()
        grid.r_time, grid.r_dt, grid.r_dt_new = self.ctx.get_time()
        if flags:
            grid.refinement, grid.i_refinements_issued = self.ctx.refinements(grid.refinement)
        if sync_state:
            self.fetch(grid)
        return grid

    def fetch(self, grid: Grid):
        out = [grid.h, grid.hu, grid.hv, grid.b]
        out = [o if (o is not None and o.flags.c_contiguous and o.dtype == np.float64) else
               np.empty(self.ctx.n_cells) for o in out]
        self.ctx.download_state(out)
        grid.h, grid.hu, grid.hv, grid.b = out
        return grid

    def close(self):
        self.ctx.close()


def initial_dt(mesh: Mesh, h, hu, hv, b, courant):
    """Initial time step of the init_dofs traversal (src/SWE/SWE_initialize.f90:325-335):
    courant * min(volume / (sum(edge sizes) * max wave speed)), with the unscaled
    cell geometry the reference uses there."""
    from .geometry import leg_sizes, volumes
    leg = leg_sizes()
    vols = volumes()
    best = np.finfo(np.float64).max
    for dd in np.unique(mesh.depth):
        sel = mesh.depth == dd
        dd = int(dd)
        edges = (leg[dd + 1] + leg[dd]) + leg[dd + 1]
        depth = h[sel] - b[sel]
        wet = depth > 0.0
        if not wet.any():
            continue
        dw = depth[wet]
        speed = np.sqrt(G * dw) + np.sqrt((hu[sel][wet] ** 2 + hv[sel][wet] ** 2) / (dw * dw))
        smax = float(speed.max())
        if smax > 0.0:
            best = min(best, vols[dd] / (edges * smax))
    return courant * best


def remesh(cfg, mesh, flags, h, hu, hv, b, bathymetry=None):
    """One remesh of the run loop: the adaption step from the time step's flags
    (swe_mesh_adapt: conformity, refine/coarsen, order-0 transfer), with refined
    cells' b integrated from `bathymetry(x, y)` when it is given (refine_op's
    get_bathymetry_at_element, src/SWE/SWE_adapt.f90:132, with _ADAPT_INTEGRATE),
    else their parent's. Returns the new mesh and (h, hu, hv, b)."""
    new, (h, hu, hv, b), src = adapt(mesh, flags, h, hu, hv, b, with_source=True)
    if bathymetry is not None and b is not None:
        from .scenarios import element_bathymetry
        fine = new.depth > mesh.depth[src]
        if fine.any():
            ver = new.vertices
            if ver is None:
                ver = mesh_from_depths(new.depth, centroids=False, vertices=True).vertices
            b[fine] = element_bathymetry(ver[fine], new.depth[fine], cfg.i_max_depth, bathymetry, cfg.scaling,
                                         cfg.offset)
    return new, (h, hu, hv, b)


def run_adaptive(cfg, mesh, h, hu, hv, b, dt, steps, adapt_every=1, bathymetry=None, device=0, time=0.0):
    """The SWE run loop with host remeshing (src/SWE/SWE.f90:378-392): step i
    (from 1) is preceded by a remesh when i % adapt_every == 0, from the
    refinement flags of the step before (swe_mesh_adapt + swe_mesh_build, then
    an upload); refined cells take b integrated from `bathymetry(x, y)` when it
    is given (get_bathymetry_at_element of refine_op, src/SWE/SWE_adapt.f90:132,
    with _ADAPT_INTEGRATE: scenarios.element_bathymetry), else their parent's. Returns the
    final (mesh, h, hu, hv, b, time, dt) and timings: device seconds of the steps
    (CUDA events) and host seconds of the remeshes and uploads."""
    import time as _time

    import torch
    ctx = SweContext(device)
    stream = torch.cuda.Stream(device=device)
    ctx.set_stream(stream.cuda_stream)
    stats = {"steps": 0, "cell_updates": 0, "step_s": 0.0, "remesh_s": 0.0, "remeshes": 0, "cells": [],
             "download_s": 0.0, "adapt_s": 0.0, "upload_s": 0.0}
    try:
        ctx.set_params(cfg.params())
        ctx.upload_mesh(mesh)
        ctx.upload_state(h, hu, hv, b)
        ctx.set_time(time, dt)
        flags = np.zeros(mesh.n_cells, np.int8)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        for i in range(1, steps + 1):
            if adapt_every > 0 and i % adapt_every == 0 and i > 1:
                t0 = _time.perf_counter()
                h, hu, hv, b = ctx.download_state()
                time, dt, _ = ctx.get_time()
                t1 = _time.perf_counter()
                mesh, (h, hu, hv, b) = remesh(cfg, mesh, flags, h, hu, hv, b, bathymetry)
                t2 = _time.perf_counter()
                ctx.upload_mesh(mesh)
                ctx.upload_state(h, hu, hv, b)
                ctx.set_time(time, dt)
                t3 = _time.perf_counter()
                stats["remesh_s"] += t3 - t0
                stats["download_s"] += t1 - t0
                stats["adapt_s"] += t2 - t1
                stats["upload_s"] += t3 - t2
                stats["remeshes"] += 1
            e0.record(stream)
            ctx.traverse(1)
            e1.record(stream)
            e1.synchronize()
            stats["step_s"] += e0.elapsed_time(e1) * 1e-3
            stats["steps"] += 1
            stats["cell_updates"] += mesh.n_cells
            stats["cells"].append(mesh.n_cells)
            flags, _ = ctx.refinements()
        h, hu, hv, b = ctx.download_state()
        time, dt, _ = ctx.get_time()
    finally:
        ctx.close()
    return (mesh, h, hu, hv, b, time, dt), stats
