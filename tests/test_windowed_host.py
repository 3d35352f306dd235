"""Host parts of the windowed adjoint: the order-0 transfer of a remesh, its
adjoint (the exact transpose), and the gauge point location on a mesh."""
import numpy as np

from samoa_gb300 import swe
from samoa_gb300.adjoint import Transfer, locate_points


def _adapted(seed=3, rounds=6):
    rng = np.random.default_rng(seed)
    mesh = swe.mesh_from_depths(np.full(2 << 6, 6, np.int8), vertices=True)
    for _ in range(rounds):
        f = rng.choice([-1, 0, 1], size=mesh.n_cells, p=[0.4, 0.3, 0.3]).astype(np.int8)
        f[mesh.depth >= 10] = np.minimum(f[mesh.depth >= 10], 0)
        mesh, _ = swe.adapt(mesh, f)
    return mesh, rng


def test_transfer_matches_adapt_and_adjoint_is_transpose(swe_lib):
    mesh, rng = _adapted()
    n = mesh.n_cells
    f = rng.choice([-1, 0, 1], size=n, p=[0.4, 0.3, 0.3]).astype(np.int8)
    q = rng.normal(size=n)
    new, (qn, _, _, _), src = swe.adapt(mesh, f, q, with_source=True)
    tr = Transfer(mesh.depth, new.depth, src)
    assert tr.merged.any() and (new.depth > mesh.depth[src]).any()  # both merges and refinements
    assert np.array_equal(tr.apply(q), qn)  # the same values as the library's transfer
    x, y = rng.normal(size=n), rng.normal(size=new.n_cells)
    assert abs(np.dot(tr.apply(x), y) - np.dot(x, tr.adjoint(y))) <= 1e-12 * np.abs(x).sum() * np.abs(y).max()


def test_locate_points_finds_the_containing_cell(swe_lib):
    mesh, rng = _adapted(seed=5)
    k = rng.choice(mesh.n_cells, 50, replace=False)
    assert np.array_equal(locate_points(mesh.vertices, mesh.centroids[k]), k)
