"""CPU tests of the oracle: mesh geometry, the parity-based Jacobi form against
the sequential walk, analytic invariants, and the exact 1-D Riemann solutions
of the reference's scripts/python/Riemann.ipynb (cells 7-13)."""
import numpy as np
import pytest
from scipy.optimize import brentq

from oracle import oracle as O
from samoa_gb300 import scenarios, swe

from .helpers import assert_state_equal, omp_state, oracle_params, walk_state

# local edge index -> (node, node), 0-based: edge i joins nodes 1+mod(i,3), 1+mod(i+1,3)
# (src/Generic/Generic_initialize.f90:151-152)
EDGE_NODES = {1: (1, 2), 2: (2, 0), 3: (0, 1)}


def test_leg_and_volume_tables(oracle_lib):
    assert O.leg_size(0) == 1.0
    assert O.leg_size(1) == np.sqrt(0.5)
    for i in range(0, 61):
        assert O.cell_volume(i) == 0.5 ** (i + 1)
        assert abs(O.leg_size(i) / (0.5 ** (i / 2.0)) - 1.0) < 1e-14
    for p in [q for q in range(-8, 9) if q]:
        for e in (1, 2, 3):
            n = O.normal(p, e)
            assert abs(np.hypot(*n) - 1.0) < 1e-15


@pytest.mark.parametrize("depth", range(0, 9))
def test_mesh_geometry(oracle_lib, depth):
    m = O.mesh_uniform(depth)
    co, c5 = m["coords"], m["cells5"]
    n = m["n"]
    assert len(m["edge_cells"]) * 2 + len(m["bnd_cell"]) == 3 * n

    def pts(c, li):
        a, b = EDGE_NODES[li]
        return co[c][a], co[c][b]

    for (c1, c2), (l1, l2) in zip(m["edge_cells"], m["edge_local"]):
        assert c1 < c2
        p1, p2 = pts(c1, l1), pts(c2, l2)
        assert {tuple(p1[0]), tuple(p1[1])} == {tuple(p2[0]), tuple(p2[1])}
        n1, n2 = O.normal(c5[c1, 2], l1), O.normal(c5[c2, 2], l2)
        assert np.array_equal(n1, -n2)
        assert np.dot(n1, (p1[0] + p1[1]) / 2 - co[c1].mean(0)) > 0
        assert abs(np.dot(n1, p1[1] - p1[0])) < 1e-15
    for c, li in zip(m["bnd_cell"], m["bnd_local"]):
        p = pts(c, li)
        on_x = p[0][0] == p[1][0] and p[0][0] in (0.0, 1.0)
        on_y = p[0][1] == p[1][1] and p[0][1] in (0.0, 1.0)
        assert on_x or on_y
        assert np.dot(O.normal(c5[c, 2], li), (p[0] + p[1]) / 2 - co[c].mean(0)) > 0
    area = 0.5 * np.abs((co[:, 1, 0] - co[:, 0, 0]) * (co[:, 2, 1] - co[:, 0, 1]) -
                        (co[:, 2, 0] - co[:, 0, 0]) * (co[:, 1, 1] - co[:, 0, 1]))
    assert area.sum() == 1.0 and np.all(area == area[0])


def _walk_vs_omp(scn, steps):
    g = scn.grid
    W = walk_state(int(g.mesh.depth[0]), g)
    S = omp_state(g.mesh, g)
    P = oracle_params(scn.cfg)
    for k in range(steps):
        W.steps(P, 1)
        S.steps(P, 1)
        assert_state_equal("step %d" % k, S.h, S.hu, S.hv, W.h, W.hu, W.hv)
        assert np.array_equal(S.flags, W.flags)
        assert S.n_refine == W.n_refine
        assert list(S.scal) == list(W.scal)


@pytest.mark.parametrize("boundary", ["outflow", "slip", "noslip"])
@pytest.mark.parametrize("solver", ["fwave", "aug_riemann", "llfbath", "lfbath"])
def test_jacobi_form_equals_walk(oracle_lib, solver, boundary):
    """The parity-based form the GPU uses (lower-numbered cell first-touched on
    even steps, legs summed in reverse on odd steps, normals of the upload
    orientation) equals the literal walk with per-step cell reversal."""
    scn = scenarios.parabolic_bowl(log2_cells=10, solver=solver, amplitude=2.0, sigma=0.08)
    scn.cfg.boundary = boundary
    _walk_vs_omp(scn, 9)


def test_jacobi_form_equals_walk_refinement(oracle_lib):
    scn = scenarios.radial_dam_break(log2_cells=10)
    scn.cfg.i_min_depth, scn.cfg.i_max_depth = 4, 12
    _walk_vs_omp(scn, 6)


def test_lake_at_rest(oracle_lib):
    scn = scenarios.lake_at_rest(log2_cells=10)
    g = scn.grid
    S = omp_state(g.mesh, g)
    S.steps(oracle_params(scn.cfg), 20)
    assert np.array_equal(S.h, g.h) and not S.hu.any() and not S.hv.any()


def test_mass_conservation(oracle_lib):
    scn = scenarios.radial_dam_break(log2_cells=10, boundary="noslip")
    g = scn.grid
    vol = O.cell_volume(int(g.mesh.depth[0]))
    m0 = np.sum(g.h - g.b) * vol
    S = omp_state(g.mesh, g)
    S.steps(oracle_params(scn.cfg), 300)
    m1 = np.sum(S.h - g.b) * vol
    assert abs(m1 - m0) / m0 < 1e-12


def test_radial_symmetry(oracle_lib):
    """The mesh is symmetric under (x, y) -> (y, x); the radial dam break stays
    symmetric with hu and hv swapped (to round-off: edge orientation differs)."""
    scn = scenarios.radial_dam_break(log2_cells=12, boundary="slip")
    g = scn.grid
    c = g.mesh.centroids
    key = np.round(c * 2 ** 20).astype(np.int64)
    idx = {tuple(k): i for i, k in enumerate(key)}
    mirror = np.array([idx[(k[1], k[0])] for k in key])
    S = omp_state(g.mesh, g)
    S.steps(oracle_params(scn.cfg), 30)
    scale = np.abs(S.hu).max()
    assert np.abs(S.h - S.h[mirror]).max() < 1e-11
    assert np.abs(S.hu - S.hv[mirror]).max() < 1e-10 * scale


def _exact_riemann(hl, hr, ul, ur, g, xi):
    """Exact 1-D dam-break solution h(x/t) (restating Riemann.ipynb cells 3-10)."""
    def phi_l(h):
        return ul + (2.0 * (np.sqrt(g * hl) - np.sqrt(g * h)) if h < hl else
                     (hl - h) * np.sqrt(g / 2.0 * (1.0 / hl + 1.0 / h)))

    def phi_r(h):
        return ur + ((h - hr) * np.sqrt(g / 2.0 * (1.0 / h + 1.0 / hr)) if h > hr else
                     2.0 * (np.sqrt(g * h) - np.sqrt(g * hr)))

    out = np.empty_like(xi)
    if hr == 0.0:  # dry bed: one rarefaction
        cl = np.sqrt(g * hl)
        s_head, s_tail = ul - cl, ul + 2.0 * cl
        fan = (ul + 2.0 * cl - xi) ** 2 / (9.0 * g)
        out[:] = np.where(xi < s_head, hl, np.where(xi < s_tail, fan, 0.0))
        return out
    hm = brentq(lambda h: phi_r(h) - phi_l(h), 1e-12, 10 * max(hl, hr))
    um = phi_l(hm)
    # left wave (rarefaction here: hl > hm), right wave (shock: hm > hr)
    s1l, s1r = ul - np.sqrt(g * hl), um - np.sqrt(g * hm)
    fan = (ul + 2.0 * np.sqrt(g * hl) - xi) ** 2 / (9.0 * g)
    s2 = (hm * um - hr * ur) / (hm - hr)
    out[:] = np.where(xi < s1l, hl, np.where(xi < s1r, fan, np.where(xi < s2, hm, hr)))
    return out


@pytest.mark.parametrize("case", [(3.0, 1.0), (1.0, 0.0)])
def test_converges_to_exact_dam_break(oracle_lib, case):
    """Riemann.ipynb test cases (hl, hr) = (3, 1) and (1, 0) with g = 9.80665:
    the L1 error of the 2-D step against the exact 1-D solution shrinks with
    resolution (f-wave; the dry case with the wet/dry fix-ups)."""
    hl, hr = case
    errs = []
    for log2 in (10, 12, 14):
        d = log2 - 1
        mesh = swe.uniform_mesh(d)
        cfg = swe.Config(flux_solver="fwave", boundary="outflow", courant_number=0.45, dry_tolerance=1e-3,
                         scaling=1.0, offset=(-0.5, -0.5), i_min_depth=d, i_max_depth=d)
        x = mesh.centroids[:, 0] - 0.5
        b = np.zeros(mesh.n_cells)
        h = np.where(x < 0.0, hl, hr)
        g0 = swe.Grid(mesh, h, np.zeros_like(h), np.zeros_like(h), b)
        g0.r_dt = swe.initial_dt(mesh, h, g0.hu, g0.hv, b, cfg.courant_number)
        S = omp_state(mesh, g0)
        P = oracle_params(cfg)
        while S.scal[0] < 0.04:
            S.steps(P, 1)
        t = S.scal[0]
        exact = _exact_riemann(hl, hr, 0.0, 0.0, 9.80665, x / t)
        errs.append(np.mean(np.abs((S.h - b) - exact)))
    if hr > 0.0:
        assert errs[1] < 0.8 * errs[0] and errs[2] < 0.8 * errs[1], errs
        assert errs[2] < 0.02 * hl, errs
    else:  # the dry front converges slowly under the wet/dry clamps, but it converges
        assert errs[2] < errs[1] < errs[0], errs
        assert errs[2] < 0.03 * hl, errs


def test_riemann_solver_branches_finite(oracle_lib):
    """Wet/dry, walls and dry/dry produce finite net updates; dry/dry gives zeros."""
    nl, nr, s = O.geoclaw_solver(O.FWAVE, 0.0, 0.0, 0, 0, 0, 0, 0, 0)
    assert not nl.any() and not nr.any() and s == 0.0
    for solver in (O.FWAVE, O.AUG_RIEMANN):
        # right side dry and higher: wall
        nl, nr, s = O.geoclaw_solver(solver, 2.0, 0.0, 1.0, 0.0, 0.5, 0.0, -2.0, 5.0)
        assert np.isfinite(nl).all() and np.isfinite(nr).all() and s > 0
        assert not nr.any()  # the wall eliminates the right-going waves
        # left dry and higher: wall on the left
        nl, nr, s = O.geoclaw_solver(solver, 0.0, 2.0, 0.0, -1.0, 0.0, 0.5, 5.0, -2.0)
        assert not nl.any() and np.isfinite(nr).all()
