"""Host remesh handoff: meshes from leaf depths and one adaption step
(conformity closure, refine/coarsen, order-0 state transfer), checked against
the oracle's walk and against the invariants of the adaption rules."""
import numpy as np
import pytest

from oracle import oracle as O
from samoa_gb300 import _lib, scenarios, swe

from .helpers import omp_state, oracle_params


def random_mesh(seed, rounds=10, dmax=14):
    rng = np.random.default_rng(seed)
    mesh = swe.mesh_from_depths(np.zeros(2, np.int8))
    for _ in range(rounds):
        f = rng.choice([-1, 0, 1], size=mesh.n_cells, p=[0.3, 0.3, 0.4]).astype(np.int8)
        f[mesh.depth >= dmax] = np.minimum(f[mesh.depth >= dmax], 0)
        mesh, _ = swe.adapt(mesh, f)
    return mesh


def assert_same_mesh(a, b):
    for k in ("depth", "plotter", "edge_cells", "edge_local", "bnd_cell", "bnd_local"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_mesh_from_depths_matches_oracle_walk(swe_lib, oracle_lib, seed):
    mesh = random_mesh(seed)
    assert len(np.unique(mesh.depth)) > 2
    o = O.mesh_from_depths(mesh.depth)
    assert np.array_equal(o["cells5"][:, 1], mesh.depth)
    assert np.array_equal(o["cells5"][:, 2], mesh.plotter)
    for k in ("edge_cells", "edge_local", "bnd_cell", "bnd_local"):
        assert np.array_equal(o[k], getattr(mesh, k)), k
    # conforming: the two cells of every inner edge share both end points
    v = o["coords"]
    for (a, b) in mesh.edge_cells:
        assert len({tuple(p) for p in v[a]} & {tuple(p) for p in v[b]}) == 2


def test_uniform_depths_give_the_uniform_mesh(swe_lib):
    u = swe.uniform_mesh(9)
    assert_same_mesh(swe.mesh_from_depths(u.depth), u)


def test_rejects_depths_that_are_no_tree(swe_lib):
    with pytest.raises(_lib.SweError):
        swe.mesh_from_depths(np.array([0, 1, 1], np.int8))    # too many leaves
    with pytest.raises(_lib.SweError):
        swe.mesh_from_depths(np.array([1, 1, 1], np.int8))    # too few
    with pytest.raises(_lib.SweError):
        swe.mesh_from_depths(np.array([0, 2, 2, 1], np.int8))  # not conforming (hanging node)


def _areas(mesh):
    return np.ldexp(1.0, -(mesh.depth.astype(int) + 1))


def test_adapt_invariants(swe_lib):
    mesh = random_mesh(7, rounds=8)
    n = mesh.n_cells
    rng = np.random.default_rng(8)
    h = rng.normal(size=n)
    # nothing flagged: nothing changes
    m0, (h0,) = (lambda r: (r[0], r[1][:1]))(swe.adapt(mesh, np.zeros(n, np.int8), h))
    assert_same_mesh(m0, mesh)
    assert np.array_equal(h0, h)
    # refine everything: every cell is split at least once (the conformity
    # closure splits some twice where a coarser neighbour meets a finer one)
    m1, (src1, _, _, _), s1 = swe.adapt(mesh, np.ones(n, np.int8), np.arange(n, dtype=np.float64), with_source=True)
    assert np.array_equal(src1.astype(np.int64), s1)
    assert np.all(m1.depth >= mesh.depth[s1] + 1)
    assert m1.n_cells >= 2 * n
    # on a uniform mesh: refine all, then coarsen all returns to the start bit for bit
    u = swe.uniform_mesh(6)
    hu_ = rng.normal(size=u.n_cells)
    mu1, (hu1, _, _, _) = swe.adapt(u, np.ones(u.n_cells, np.int8), hu_)
    assert_same_mesh(mu1, swe.uniform_mesh(7))
    mu2, (hu2, _, _, _) = swe.adapt(mu1, -np.ones(mu1.n_cells, np.int8), hu1)
    assert_same_mesh(mu2, u)
    assert np.array_equal(hu2, hu_)
    # random flags: the area integral of the state is kept (copy / average)
    f = rng.choice([-1, 0, 1], size=n, p=[0.5, 0.2, 0.3]).astype(np.int8)
    m3, (h3, _, _, _) = swe.adapt(mesh, f, h)
    assert abs(np.sum(h3 * _areas(m3)) - np.sum(h * _areas(mesh))) < 1e-13 * np.sum(np.abs(h) * _areas(mesh))
    assert np.isclose(_areas(m3).sum(), 1.0)
    # every refinement request is honoured: a flagged cell's area is split
    m4, (src,) = (lambda r: (r[0], r[1][:1]))(swe.adapt(mesh, f, np.arange(n, dtype=np.float64)))
    refined = np.unique(src[m4.depth > mesh.depth[src.astype(int)]].astype(int))
    assert set(np.nonzero(f == 1)[0]) <= set(refined)


def test_coarsening_needs_both_siblings(swe_lib):
    mesh = swe.uniform_mesh(4)
    n = mesh.n_cells
    f = np.zeros(n, np.int8)
    f[0] = -1  # its sibling keeps: no change
    m, _ = swe.adapt(mesh, f)
    assert_same_mesh(m, mesh)
    f[:] = -1  # all: the uniform mesh one level up
    m, _ = swe.adapt(mesh, f)
    assert_same_mesh(m, swe.uniform_mesh(3))


def test_apriori_dam_break_mesh(swe_lib):
    scn = scenarios.adaptive_dam_break(min_depth=6, max_depth=12)
    d = scn.grid.mesh.depth
    assert d.min() == 6 and d.max() == 12
    # the finest cells sit on the step x = 0
    c = scn.grid.mesh.centroids
    assert np.abs(c[d == 12, 0] - 0.5).max() < 0.05 and np.abs(c[d == 6, 0] - 0.5).min() > 0.05


def test_jacobi_form_equals_walk_on_adaptive_mesh(oracle_lib, swe_lib):
    scn = scenarios.adaptive_dam_break(min_depth=5, max_depth=10)
    g = scn.grid
    o = O.mesh_from_depths(g.mesh.depth)
    P = oracle_params(scn.cfg)
    W = O.WalkState(o["cells5"], g.h, g.hu, g.hv, g.b, g.r_time, g.r_dt)
    S = omp_state(g.mesh, g)
    for k in range(6):
        W.steps(P, 1)
        S.steps(P, 1)
        assert np.array_equal(W.h, S.h) and np.array_equal(W.hu, S.hu) and np.array_equal(W.hv, S.hv), k
        assert np.array_equal(W.flags, S.flags), k
        assert W.dt == float(S.scal[1]), k
