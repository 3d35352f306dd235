"""ctypes front end of the oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
may import this module, and only as the reference results are compared with. It wraps ``swe_oracle.c``, the
strict-IEEE C restatement of sam(oa)^2's SWE Euler step, and ``swe_oracle_adapt.c``,
the restatement of one adaption step and of the integrated bathymetry.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None


class Params(C.Structure):
    """Mirror of the oracle's parameter block (same layout as swe_params in include/samoa_swe.h)."""
    _fields_ = [("solver", C.c_int32), ("bc", C.c_int32), ("dry_tolerance", C.c_double),
                ("courant", C.c_double), ("scaling", C.c_double), ("min_depth", C.c_int32),
                ("max_depth", C.c_int32), ("max_time", C.c_double), ("output_time_step", C.c_double)]


FWAVE, AUG_RIEMANN, LF, LF_BATH, LLF, LLF_BATH = 1, 3, 10, 11, 12, 13
BC_OUTFLOW, BC_SLIP, BC_NOSLIP = 0, 1, 2


def lib():
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            path = _build.build()
        L = C.CDLL(path)
        P = C.c_void_p
        i64, i32, dbl = C.c_int64, C.c_int, C.c_double
        L.oracle_leg_size.restype = dbl
        L.oracle_leg_size.argtypes = [i32]
        L.oracle_cell_volume.restype = dbl
        L.oracle_cell_volume.argtypes = [i32]
        L.oracle_normal.argtypes = [i32, i32, P]
        L.oracle_mesh_uniform.restype = i64
        L.oracle_mesh_uniform.argtypes = [i32, P, P]
        L.oracle_mesh_from_depths.restype = i64
        L.oracle_mesh_from_depths.argtypes = [i64, P, P, P]
        L.oracle_mesh_edges.restype = i32
        L.oracle_mesh_edges.argtypes = [P, i64, P, P, P, P, P, P]
        L.oracle_geoclaw_solver.argtypes = [i32] + [dbl] * 10 + [P, P, P]
        L.oracle_edge_flux.argtypes = [i32, P, P, P, dbl, P, P]
        L.oracle_steps.restype = i32
        L.oracle_steps.argtypes = [P, i64, P, P, P, P, P, P, P, P, i64, P, P]
        L.oracle_steps_omp.restype = i32
        L.oracle_steps_omp.argtypes = [P, i64, P, P, i64, P, P, i64, P, P, P, P, P, P, P, P, P, P, P, P,
                                       P, i64, P, P, P, i32]
        L.oracle_cell_slots.restype = i32
        L.oracle_cell_slots.argtypes = [i64, i64, P, P, i64, P, P, P]
        L.oracle_max_threads.restype = i32
        L.oracle_bathymetry_cells.restype = i32
        L.oracle_bathymetry_cells.argtypes = [i64, P, P, P]
        L.oracle_adapt.restype = i64
        L.oracle_adapt.argtypes = [i64, P, P, P, P, P, P, P, i64, P, P, P, P, P, P]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def leg_size(i):
    return lib().oracle_leg_size(i)


def cell_volume(i):
    return lib().oracle_cell_volume(i)


def normal(plotter, edge_index):
    out = np.zeros(2)
    lib().oracle_normal(plotter, edge_index, _p(out))
    return out


def mesh_uniform(depth):
    """Uniform Sierpinski mesh of the unit square, reference depth ``depth`` (2^(depth+1) cells).

    Returns dict with cells5 (int8[n,5]: entity, depth, plotter, turtle, colour),
    coords (float64[n,3,2]) and the edge streams.
    """
    n = 1 << (depth + 1)
    cells5 = np.zeros((n, 5), np.int8)
    coords = np.zeros((n, 3, 2), np.float64)
    got = lib().oracle_mesh_uniform(depth, _p(cells5), _p(coords))
    assert got == n
    m = dict(n=n, cells5=cells5, coords=coords)
    m.update(mesh_edges(cells5))
    return m


def mesh_from_depths(depths):
    """Mesh of the tree whose leaves in traversal order have these depths (an
    adaptive conforming mesh); same outputs as mesh_uniform."""
    d = np.ascontiguousarray(depths, np.int8)
    n = len(d)
    cells5 = np.zeros((n, 5), np.int8)
    coords = np.zeros((n, 3, 2), np.float64)
    got = lib().oracle_mesh_from_depths(n, _p(d), _p(cells5), _p(coords))
    if got != n:
        raise RuntimeError("oracle_mesh_from_depths failed: %d" % got)
    m = dict(n=n, cells5=cells5, coords=coords)
    m.update(mesh_edges(cells5))
    return m


def mesh_edges(cells5):
    n = cells5.shape[0]
    cap = 2 * n + 8
    ec = np.zeros((cap, 2), np.int64)
    el = np.zeros((cap, 2), np.int8)
    bc = np.zeros(n + 8, np.int64)
    bl = np.zeros(n + 8, np.int8)
    ne = np.zeros(1, np.int64)
    nb = np.zeros(1, np.int64)
    rc = lib().oracle_mesh_edges(_p(np.ascontiguousarray(cells5)), n, _p(ec), _p(el), _p(ne), _p(bc), _p(bl),
                                 _p(nb))
    if rc != 0:
        raise RuntimeError("oracle_mesh_edges failed: %d" % rc)
    ne, nb = int(ne[0]), int(nb[0])
    return dict(edge_cells=ec[:ne].copy(), edge_local=el[:ne].copy(), bnd_cell=bc[:nb].copy(),
                bnd_local=bl[:nb].copy())


def cell_slots(n, edge_cells, edge_local, bnd_cell, bnd_local):
    out = np.zeros(3 * n, np.int64)
    rc = lib().oracle_cell_slots(n, len(edge_cells), _p(np.ascontiguousarray(edge_cells, np.int64)),
                                 _p(np.ascontiguousarray(edge_local, np.int8)), len(bnd_cell),
                                 _p(np.ascontiguousarray(bnd_cell, np.int64)),
                                 _p(np.ascontiguousarray(bnd_local, np.int8)), _p(out))
    if rc != 0:
        raise RuntimeError("inconsistent edge streams")
    return out


def make_params(solver=FWAVE, bc=BC_OUTFLOW, dry_tolerance=0.01, courant=0.5, scaling=1.0, min_depth=0,
                max_depth=14, max_time=-1.0, output_time_step=-1.0):
    return Params(solver, bc, dry_tolerance, courant, scaling, min_depth, max_depth, max_time,
                  output_time_step)


def geoclaw_solver(solver, hL, hR, huL, huR, hvL, hvR, bL, bR, drytol=0.01, g=9.80665):
    nl, nr, ms = np.zeros(3), np.zeros(3), np.zeros(1)
    lib().oracle_geoclaw_solver(solver, hL, hR, huL, huR, hvL, hvR, bL, bR, drytol, g, _p(nl), _p(nr), _p(ms))
    return nl, nr, float(ms[0])


def edge_flux(solver, normal_, qL, qR, drytol=0.01):
    n = np.ascontiguousarray(normal_, np.float64)
    a = np.ascontiguousarray(qL, np.float64)
    b = np.ascontiguousarray(qR, np.float64)
    ul, ur = np.zeros(4), np.zeros(4)
    lib().oracle_edge_flux(solver, _p(n), _p(a), _p(b), drytol, _p(ul), _p(ur))
    return ul, ur


class WalkState:
    """State of the sequential (reference-order) oracle: per-cell types reversed in place each step."""

    def __init__(self, cells5, h, hu, hv, b, time=0.0, dt=0.0):
        self.cells5 = np.ascontiguousarray(cells5, np.int8).copy()
        self.n = self.cells5.shape[0]
        self.reversed = C.c_int(0)
        self.h = np.ascontiguousarray(h, np.float64).copy()
        self.hu = np.ascontiguousarray(hu, np.float64).copy()
        self.hv = np.ascontiguousarray(hv, np.float64).copy()
        self.b = np.ascontiguousarray(b, np.float64).copy()
        self.flags = np.zeros(self.n, np.int8)
        self.scal = np.array([time, dt], np.float64)
        self.n_refine = 0
        self.dt_new = 0.0

    @property
    def time(self):
        return float(self.scal[0])

    @property
    def dt(self):
        return float(self.scal[1])

    def steps(self, params, k=1):
        nr = np.zeros(1, np.int64)
        dn = np.zeros(1, np.float64)
        rc = lib().oracle_steps(C.byref(params), self.n, _p(self.cells5), C.byref(self.reversed), _p(self.h),
                                _p(self.hu), _p(self.hv), _p(self.b), _p(self.flags), _p(self.scal), k, _p(nr),
                                _p(dn))
        if rc != 0:
            raise RuntimeError("oracle_steps failed: %d" % rc)
        self.n_refine = int(nr[0])
        self.dt_new = float(dn[0])


class OmpState:
    """State of the OpenMP oracle over the C-ABI mesh format (upload order, parity-based orientation)."""

    def __init__(self, depth, plotter, edge_cells, edge_local, bnd_cell, bnd_local, h, hu, hv, b, time=0.0,
                 dt=0.0, parity=0):
        self.n = len(depth)
        self.depth = np.ascontiguousarray(depth, np.int8)
        self.plotter = np.ascontiguousarray(plotter, np.int8)
        self.edge_cells = np.ascontiguousarray(edge_cells, np.int64)
        self.edge_local = np.ascontiguousarray(edge_local, np.int8)
        self.bnd_cell = np.ascontiguousarray(bnd_cell, np.int64)
        self.bnd_local = np.ascontiguousarray(bnd_local, np.int8)
        self.slots = cell_slots(self.n, self.edge_cells, self.edge_local, self.bnd_cell, self.bnd_local)
        self.h = np.ascontiguousarray(h, np.float64).copy()
        self.hu = np.ascontiguousarray(hu, np.float64).copy()
        self.hv = np.ascontiguousarray(hv, np.float64).copy()
        self.b = np.ascontiguousarray(b, np.float64).copy()
        self._ho = np.empty_like(self.h)
        self._huo = np.empty_like(self.h)
        self._hvo = np.empty_like(self.h)
        self.flags = np.zeros(self.n, np.int8)
        self.scal = np.array([time, dt], np.float64)
        self.parity = np.array([parity], np.int64)
        self.buf = np.empty(8 * len(self.edge_cells) + 4 * len(self.bnd_cell) + 1, np.float64)
        self.n_refine = 0
        self.dt_new = 0.0

    def steps(self, params, k=1, threads=0):
        nr = np.zeros(1, np.int64)
        dn = np.zeros(1, np.float64)
        L = lib()
        rc = L.oracle_steps_omp(C.byref(params), self.n, _p(self.depth), _p(self.plotter), len(self.edge_cells),
                                _p(self.edge_cells), _p(self.edge_local), len(self.bnd_cell), _p(self.bnd_cell),
                                _p(self.bnd_local), _p(self.slots), _p(self.h), _p(self.hu), _p(self.hv),
                                _p(self.b), _p(self._ho), _p(self._huo), _p(self._hvo), _p(self.flags),
                                _p(self.scal), _p(self.parity), k, _p(self.buf), _p(nr), _p(dn), threads)
        if rc != 0:
            raise RuntimeError("oracle_steps_omp failed: %d" % rc)
        self.n_refine = int(nr[0])
        self.dt_new = float(dn[0])


def max_threads():
    return lib().oracle_max_threads()


BATHYMETRY_KINDS = {"flat": 0, "bowl": 1}


def bath_spec(kind, p0, p1=0.0, scaling=1.0, offset=(0.0, 0.0), max_depth=0):
    """The bathymetry the oracle samples: "flat" (constant p0) or "bowl"
    (-p0 * (1 - r^2 / p1^2)), world coordinates scaling * x + offset, integrated
    over 2^min(16, max_depth - depth) sub-triangles of a cell."""
    return np.array([BATHYMETRY_KINDS[kind], p0, p1, scaling, offset[0], offset[1], max_depth], np.float64)


def bathymetry_cells(depths, spec):
    """get_bathymetry_at_element of every leaf of the tree with these depths."""
    d = np.ascontiguousarray(depths, np.int8)
    out = np.empty(len(d), np.float64)
    rc = lib().oracle_bathymetry_cells(len(d), _p(d), _p(np.ascontiguousarray(spec, np.float64)), _p(out))
    if rc != 0:
        raise RuntimeError("oracle_bathymetry_cells failed: %d" % rc)
    return out


def adapt(depths, flags, h=None, hu=None, hv=None, b=None, spec=None):
    """One adaption step (conformity, refine/coarsen, order-0 transfer; refined
    cells' b integrated from `spec` when given, else copied). Returns
    (depth, source, [h, hu, hv, b]) with None for the state not given."""
    d = np.ascontiguousarray(depths, np.int8)
    f = np.ascontiguousarray(flags, np.int8)
    n = len(d)
    ins = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (h, hu, hv, b)]
    cap = 4 * n
    dout = np.empty(cap, np.int8)
    src = np.empty(cap, np.int64)
    outs = [None if a is None else np.empty(cap, np.float64) for a in ins]
    q = lambda a: None if a is None else _p(a)
    sp = None if spec is None else np.ascontiguousarray(spec, np.float64)
    m = lib().oracle_adapt(n, _p(d), _p(f), *[q(a) for a in ins], q(sp), cap, _p(dout), _p(src),
                           *[q(a) for a in outs])
    if m < 0:
        raise RuntimeError("oracle_adapt failed: %d" % m)
    return dout[:m].copy(), src[:m].copy(), [None if a is None else a[:m].copy() for a in outs]
