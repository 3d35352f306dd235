"""The product's host adaptivity against the oracle's own restatement (CPU).

The oracle (oracle/swe_oracle_adapt.c) rebuilds the tree from the leaf depths
with exact integer vertices, finds edges by their midpoints and keeps the
conformity flags per cell side, merged in passes as the reference's
conformity traversals do (src/Conformity/Conformity.f90:172-314,1244-1331);
the product (swe_mesh_adapt) works on shared edge records of its own mesh
builder. Random flag sets on mixed-depth trees must give the same new leaf
depths, source cells and transferred state bit for bit, and the integrated
bathymetry (get_bathymetry_at_element with _ADAPT_INTEGRATE,
src/SWE/SWE_initialize.f90:105-147) the same b.
"""
import numpy as np
import pytest

from oracle import oracle as O
from samoa_gb300 import scenarios, swe


def _random_flags(rng, depth, lo=2, hi=14, p=(0.45, 0.3, 0.25)):
    f = rng.choice(np.array([-1, 0, 1], np.int8), size=len(depth), p=p).astype(np.int8)
    f[depth <= lo] = np.maximum(f[depth <= lo], 0)
    f[depth >= hi] = np.minimum(f[depth >= hi], 0)
    return f


def _compare(mesh, flags, state):
    new, outs, src = swe.adapt(mesh, flags, *state, with_source=True)
    d, s, o = O.adapt(mesh.depth, flags, *state)
    assert np.array_equal(new.depth, d), "leaf depths differ"
    assert np.array_equal(src, s), "source cells differ"
    for name, x, y in zip(("h", "hu", "hv", "b"), outs, o):
        assert np.array_equal(x, y), name + " differs"
    return new, outs


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_adapt_matches_oracle_on_random_flags(oracle_lib, swe_lib, seed):
    rng = np.random.default_rng(seed)
    mesh = swe.uniform_mesh(5 + seed)
    state = [rng.normal(size=mesh.n_cells) for _ in range(4)]
    seen = set()
    for _ in range(10):
        flags = _random_flags(rng, mesh.depth)
        mesh, state = _compare(mesh, flags, state)
        seen.update(np.unique(mesh.depth).tolist())
    assert len(seen) >= 6  # mixed depths were exercised


@pytest.mark.parametrize("fill", [-1, 0, 1])
def test_adapt_matches_oracle_on_uniform_flags(oracle_lib, swe_lib, fill):
    rng = np.random.default_rng(7)
    mesh = swe.uniform_mesh(6)
    for _ in range(3):
        mesh, _ = swe.adapt(mesh, _random_flags(rng, mesh.depth))
    state = [rng.normal(size=mesh.n_cells) for _ in range(4)]
    flags = np.full(mesh.n_cells, fill, np.int8)
    _compare(mesh, flags, state)


def test_adapt_without_state_and_the_two_roots(oracle_lib, swe_lib):
    mesh = swe.uniform_mesh(0)  # the two root cells: they never coarsen
    for fill in (-1, 0, 1):
        flags = np.full(2, fill, np.int8)
        new, _ = swe.adapt(mesh, flags)
        d, _, _ = O.adapt(mesh.depth, flags)
        assert np.array_equal(new.depth, d)


def test_oracle_rejects_bad_trees_and_flags(oracle_lib):
    # the first root refined twice, the second not: a hanging node on the diagonal
    with pytest.raises(RuntimeError, match="-5"):
        O.adapt(np.array([2, 2, 2, 2, 0], np.int8), np.zeros(5, np.int8))
    with pytest.raises(RuntimeError, match="-[123]"):  # not the leaves of a tree
        O.adapt(np.array([1, 1, 1], np.int8), np.zeros(3, np.int8))
    with pytest.raises(RuntimeError, match="-4"):
        O.adapt(np.array([1, 1, 1, 1], np.int8), np.array([0, 2, 0, 0], np.int8))


def _mixed_mesh(seed, rounds=6, start=5):
    rng = np.random.default_rng(seed)
    mesh = swe.uniform_mesh(start)
    for _ in range(rounds):
        mesh, _ = swe.adapt(mesh, _random_flags(rng, mesh.depth, p=(0.3, 0.3, 0.4)))
    return swe.mesh_from_depths(mesh.depth, vertices=True)


@pytest.mark.parametrize("extra", [0, 3, 9])
def test_integrated_bathymetry_matches_oracle(oracle_lib, swe_lib, extra):
    mesh = _mixed_mesh(2)
    D = int(mesh.depth.max()) + extra
    b = scenarios.element_bathymetry(mesh.vertices, mesh.depth, D, scenarios.bowl_bathymetry, 1.0, (-0.5, -0.5))
    ref = O.bathymetry_cells(mesh.depth, O.bath_spec("bowl", 10.0, 0.4, 1.0, (-0.5, -0.5), D))
    assert np.array_equal(b, ref)


def test_integration_depth_is_capped_at_16_levels(oracle_lib, swe_lib):
    mesh = swe.mesh_from_depths(np.zeros(2, np.int8), vertices=True)
    spec16 = O.bath_spec("bowl", 10.0, 0.4, 1.0, (-0.5, -0.5), 16)
    spec30 = O.bath_spec("bowl", 10.0, 0.4, 1.0, (-0.5, -0.5), 30)
    assert np.array_equal(O.bathymetry_cells(mesh.depth, spec16), O.bathymetry_cells(mesh.depth, spec30))
    b = scenarios.element_bathymetry(mesh.vertices, mesh.depth, 30, scenarios.bowl_bathymetry, 1.0, (-0.5, -0.5))
    assert np.array_equal(b, O.bathymetry_cells(mesh.depth, spec30))


def test_remesh_with_integrated_bathymetry_matches_oracle(oracle_lib, swe_lib):
    """The run loop's remesh (swe.remesh): refined cells take the integrated b,
    merged cells the mean, the rest their own; against oracle_adapt with the
    same bathymetry."""
    rng = np.random.default_rng(11)
    cfg = swe.Config(scaling=1.0, offset=(-0.5, -0.5), i_min_depth=4, i_max_depth=13)
    mesh = _mixed_mesh(3, rounds=4)
    b = scenarios.element_bathymetry(mesh.vertices, mesh.depth, cfg.i_max_depth, scenarios.bowl_bathymetry,
                                     cfg.scaling, cfg.offset)
    spec = O.bath_spec("bowl", 10.0, 0.4, cfg.scaling, cfg.offset, cfg.i_max_depth)
    assert np.array_equal(b, O.bathymetry_cells(mesh.depth, spec))
    state = [rng.normal(size=mesh.n_cells) for _ in range(3)] + [b]
    for _ in range(5):
        flags = _random_flags(rng, mesh.depth, lo=cfg.i_min_depth, hi=cfg.i_max_depth)
        new, outs = swe.remesh(cfg, mesh, flags, *state, bathymetry=scenarios.bowl_bathymetry)
        d, _, o = O.adapt(mesh.depth, flags, *state, spec=spec)
        assert np.array_equal(new.depth, d)
        for name, x, y in zip(("h", "hu", "hv", "b"), outs, o):
            assert np.array_equal(x, y), name
        mesh, state = new, outs


def test_adaptive_bowl_scenario_bathymetry_matches_oracle(oracle_lib, swe_lib):
    scn = scenarios.adaptive_bowl(min_depth=4, max_depth=9)
    m, cfg = scn.grid.mesh, scn.cfg
    spec = O.bath_spec("bowl", 10.0, 0.4, cfg.scaling, cfg.offset, cfg.i_max_depth)
    assert np.array_equal(scn.grid.b, O.bathymetry_cells(m.depth, spec))
    uni = scenarios.parabolic_bowl(log2_cells=9)
    spec = O.bath_spec("bowl", 10.0, 0.4, uni.cfg.scaling, uni.cfg.offset, uni.cfg.i_max_depth)
    assert np.array_equal(uni.grid.b, O.bathymetry_cells(uni.grid.mesh.depth, spec))
