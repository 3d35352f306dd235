"""swe_step_noalloc: the step for callers that cannot allocate device memory.

Such a caller owns all device buffers (for example a host code that takes all
its device memory from its own pool, or one that steps where an allocation would
synchronise the device); the entry point keeps its scratch in a fixed array
inside the library. These tests drive it through the C ABI on buffers the test
allocates with torch, for two calls in a row (parity 0, then 1), and check each
call's state, flags, dt_new and refinement count against the context-based
entry point (swe_traverse) on the same inputs: the arithmetic is the same, so
they must agree bit for bit. They cover every solver, the three boundary
conditions, a mixed-depth mesh, and invalid meshes (an index out of range, a
slot claimed twice and another never), each followed by a valid call that must
again match. Collected last, so a failure here comes after every other test
has run.
"""
import ctypes as C

import numpy as np
import pytest

from samoa_gb300 import _lib, scenarios, swe

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _context_steps(mesh, grid, params, steps=2):
    """The context entry point: `steps` steps, state and scalars after each."""
    ctx = swe.SweContext(0)
    try:
        ctx.set_params(params)
        ctx.upload_mesh(mesh)
        ctx.upload_state(grid.h, grid.hu, grid.hv, grid.b)
        ctx.set_time(0.0, grid.r_dt)
        ref = []
        for _ in range(steps):
            _, dt, _ = ctx.get_time()
            ctx.traverse(1)
            ctx.synchronize()
            h, hu, hv, _ = ctx.download_state()
            flags, nref = ctx.refinements()
            _, _, dt_new = ctx.get_time()
            ref.append((dt, h, hu, hv, flags.copy(), nref, dt_new))
        return ref
    finally:
        ctx.close()


class _NoAlloc:
    """Device copies of one mesh and state, and one call of the entry point."""

    def __init__(self, mesh, grid, edge_cells=None, edge_local=None):
        import torch
        self.torch = torch
        dev = torch.device("cuda", 0)
        t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
        ec = mesh.edge_cells if edge_cells is None else edge_cells
        el = mesh.edge_local if edge_local is None else edge_local
        self.n = mesh.n_cells
        self.n_edges = len(ec)
        self.n_bnd = len(mesh.bnd_cell)
        self.depth = t(mesh.depth, torch.int8)
        self.plotter = t(mesh.plotter, torch.int8)
        self.ec = t(ec.reshape(-1), torch.int64)
        self.el = t(el.reshape(-1), torch.int8)
        self.bc = t(mesh.bnd_cell, torch.int64)
        self.bl = t(mesh.bnd_local, torch.int8)
        self.state = [t(grid.h, torch.float64), t(grid.hu, torch.float64), t(grid.hv, torch.float64)]
        self.b = t(grid.b, torch.float64)
        self.out = [torch.empty(self.n, dtype=torch.float64, device=dev) for _ in range(3)]
        self.flags = torch.empty(self.n, dtype=torch.int8, device=dev)
        self.dt_new = torch.empty(1, dtype=torch.float64, device=dev)
        self.nref = torch.empty(1, dtype=torch.int64, device=dev)
        self.stream = torch.cuda.current_stream(dev).cuda_stream

    def call(self, params, dt, parity):
        rc = _lib.load().swe_step_noalloc(
            C.byref(params), self.n, _ptr(self.depth), _ptr(self.plotter), self.n_edges, _ptr(self.ec),
            _ptr(self.el), self.n_bnd, _ptr(self.bc), _ptr(self.bl), _ptr(self.state[0]), _ptr(self.state[1]),
            _ptr(self.state[2]), _ptr(self.b), _ptr(self.out[0]), _ptr(self.out[1]), _ptr(self.out[2]),
            _ptr(self.flags), C.c_double(dt), parity, _ptr(self.dt_new), _ptr(self.nref), C.c_void_p(self.stream))
        _lib.check(rc)
        self.torch.cuda.synchronize()
        return int(self.nref.item())

    def check(self, k, ref):
        _, h, hu, hv, f, nr, dn = ref
        for name, got, want in zip(("h", "hu", "hv"), self.out, (h, hu, hv)):
            assert np.isfinite(want).all(), "call %d: the context step's %s is not finite" % (k, name)
            assert np.array_equal(got.cpu().numpy(), want), "call %d: %s differs" % (k, name)
        assert np.array_equal(self.flags.cpu().numpy(), f), "call %d: flags differ" % k
        assert int(self.nref.item()) == nr, "call %d: refinement count" % k
        assert float(self.dt_new.item()) == dn, "call %d: dt_new" % k

    def advance(self):
        self.state, self.out = self.out, self.state


def _run_and_compare(mesh, grid, params, steps=2):
    ref = _context_steps(mesh, grid, params, steps)
    na = _NoAlloc(mesh, grid)
    for k in range(steps):
        na.call(params, ref[k][0], k)
        na.check(k, ref[k])
        na.advance()
    return ref


CASES = [("fwave", "outflow"), ("aug_riemann", "outflow"), ("lf", "outflow"), ("lfbath", "outflow"),
         ("llf", "outflow"), ("llfbath", "outflow"), ("fwave", "slip"), ("fwave", "noslip"),
         ("aug_riemann", "noslip"), ("llfbath", "slip")]


def _scenario(solver, boundary):
    """A uniform 2^12-cell wet/dry bowl with a moving bump; for the two LF fluxes
    without bathymetry terms, which assume b = 0 (src/SWE/SWE_euler_timestep.f90:423)
    and, for the global one, a fixed alpha of 100 m/s, a dam break over a flat
    bottom at Courant 0.05."""
    if solver in ("lf", "llf"):
        scn = scenarios.radial_dam_break(log2_cells=12, boundary=boundary, solver=solver)
        g = scn.grid
        g.b[:] = 0.0
        g.h[:] = g.h + 10.0
        scn.cfg.courant_number = 0.05
        scn.cfg.i_min_depth, scn.cfg.i_max_depth = 6, 13
        g.r_dt = swe.initial_dt(g.mesh, g.h, g.hu, g.hv, g.b, scn.cfg.courant_number)
        return scn
    scn = scenarios.parabolic_bowl(log2_cells=12, solver=solver, amplitude=2.0, sigma=0.08, min_depth=6,
                                   max_depth=13)
    scn.cfg.boundary = boundary
    return scn


@pytest.mark.parametrize("solver,boundary", CASES)
def test_noalloc_step_matches_context_step(swe_lib, solver, boundary):
    """Every solver, every boundary condition."""
    scn = _scenario(solver, boundary)
    _run_and_compare(scn.grid.mesh, scn.grid, scn.cfg.params())


def test_noalloc_mixed_depth_mesh(swe_lib):
    """The a-priori refined dam break (depths 6..12): edges between cells of
    different depths, per-cell volumes in the CFL time step."""
    scn = scenarios.adaptive_dam_break(min_depth=6, max_depth=12, solver="aug_riemann")
    m = scn.grid.mesh
    assert len(np.unique(m.depth)) > 2 and m.n_cells <= 1 << 16
    _run_and_compare(m, scn.grid, scn.cfg.params())


def _bad_meshes(m):
    """Two invalid variants of a mesh's inner-edge streams with the right counts:
    a cell index out of range, and one (cell, local edge) slot claimed twice while
    another is claimed by no edge."""
    n = m.n_cells
    ec_oob = m.edge_cells.copy()
    ec_oob[len(ec_oob) // 2, 1] = n
    el_dup = m.edge_local.copy()
    a, la = int(m.edge_cells[0, 0]), int(m.edge_local[0, 0])
    other = [int(m.edge_local[j, s]) for j in range(1, len(m.edge_cells)) for s in (0, 1)
             if int(m.edge_cells[j, s]) == a and int(m.edge_local[j, s]) != la]
    other += [int(l) for c, l in zip(m.bnd_cell, m.bnd_local) if int(c) == a and int(l) != la]
    el_dup[0, 0] = other[0]
    return [("index out of range", ec_oob, m.edge_local), ("slot claimed twice", m.edge_cells, el_dup)]


def test_noalloc_invalid_mesh_reports_and_next_call_is_clean(swe_lib):
    """An invalid mesh is reported as -1 refinements instead of stepping on what an
    earlier call left in the scratch; the call after it, on a valid mesh, matches
    the context step again (the error and the claim counts were cleared)."""
    scn = scenarios.parabolic_bowl(log2_cells=12, solver="fwave", amplitude=2.0, sigma=0.08, min_depth=6,
                                   max_depth=13)
    m, g, params = scn.grid.mesh, scn.grid, scn.cfg.params()
    ref = _context_steps(m, g, params, 1)
    good = _NoAlloc(m, g)
    good.call(params, ref[0][0], 0)  # fills the scratch slots with this mesh's updates
    good.check(0, ref[0])
    for what, ec, el in _bad_meshes(m):
        bad = _NoAlloc(m, g, edge_cells=ec, edge_local=el)
        assert bad.call(params, ref[0][0], 0) == -1, what
        good = _NoAlloc(m, g)
        good.call(params, ref[0][0], 0)
        good.check(0, ref[0])


def test_noalloc_rejects_oversized_mesh(swe_lib):
    params = swe.Config().params()
    rc = _lib.load().swe_step_noalloc(C.byref(params), 1 << 17, *([None] * 2), 0, None, None, 3 << 17, None, None,
                                      *([None] * 8), C.c_double(0.1), 0, None, None, None)
    assert rc == -1 and "65536" in _lib.last_error()
    # 2 * (2^63 - 1) + 14 wraps to 12 = 3 * 4 in 64-bit arithmetic: the counts are
    # bounded before they are added, so this is rejected
    rc = _lib.load().swe_step_noalloc(C.byref(params), 4, *([None] * 2), (1 << 63) - 1, None, None, 14,
                                      None, None, *([None] * 8), C.c_double(0.1), 0, None, None, None)
    assert rc == -1 and "inconsistent" in _lib.last_error()
