"""Shared helpers of the parity tests: run a scenario on the GPU (through the C
ABI) and on the oracle, and compare bit for bit."""
import numpy as np

from oracle import oracle as O
from samoa_gb300 import swe


def oracle_params(cfg):
    return O.make_params(solver=swe.SOLVERS[cfg.flux_solver], bc=swe.BOUNDARIES[cfg.boundary],
                         dry_tolerance=cfg.dry_tolerance, courant=cfg.courant_number, scaling=cfg.scaling,
                         min_depth=cfg.i_min_depth, max_depth=cfg.i_max_depth, max_time=cfg.r_max_time,
                         output_time_step=cfg.r_output_time_step)


def walk_state(mesh_depth, grid):
    """Oracle walk over the reference's cell grammar for a uniform mesh."""
    om = O.mesh_uniform(mesh_depth)
    return O.WalkState(om["cells5"], grid.h, grid.hu, grid.hv, grid.b, grid.r_time, grid.r_dt)


def omp_state(mesh, grid, parity=0):
    return O.OmpState(mesh.depth, mesh.plotter, mesh.edge_cells, mesh.edge_local, mesh.bnd_cell, mesh.bnd_local,
                      grid.h, grid.hu, grid.hv, grid.b, grid.r_time, grid.r_dt, parity)


def same_bits(a, b):
    """Equal as values (so +0.0 == -0.0), NaN nowhere."""
    a = np.asarray(a)
    b = np.asarray(b)
    return a.shape == b.shape and not np.isnan(a).any() and not np.isnan(b).any() and bool(np.all(a == b))


def assert_state_equal(tag, h, hu, hv, ref_h, ref_hu, ref_hv):
    for name, x, y in (("h", h, ref_h), ("hu", hu, ref_hu), ("hv", hv, ref_hv)):
        if not same_bits(x, y):
            d = np.abs(np.asarray(x) - np.asarray(y))
            i = int(np.nanargmax(d))
            raise AssertionError("%s: %s differs at %d cells, max |diff| %.3e at cell %d (%r vs %r)" %
                                 (tag, name, int((d != 0).sum()), float(d[i]), i, float(x[i]), float(y[i])))


def rel_l2(a, b):
    den = max(float(np.linalg.norm(b)), 1e-300)
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b))) / den


def random_states_scenario(solver, seed=5, depth=9):
    """Random wet states on a uniform mesh: shocks, rarefactions and mixed waves on
    every edge kind (every branch of the augmented solver's riemanntype), about
    5 % dry cells, outflow walls."""
    from samoa_gb300 import scenarios, swe
    mesh = swe.uniform_mesh(depth)
    n = mesh.n_cells
    rng = np.random.default_rng(seed)
    b = rng.uniform(-12.0, -2.0, n)
    d = rng.uniform(0.5, 10.0, n) * (rng.random(n) > 0.05)
    h = b + d
    hu = rng.normal(0.0, 6.0, n) * d
    hv = rng.normal(0.0, 6.0, n) * d
    cfg = swe.Config(flux_solver=solver, boundary="outflow", courant_number=0.3, dry_tolerance=1e-3, scaling=1.0,
                     offset=(-0.5, -0.5), i_min_depth=max(depth - 1, 0), i_max_depth=depth + 1)
    dt = swe.initial_dt(mesh, h, hu, hv, b, cfg.courant_number)
    return scenarios.Scenario("random", swe.Grid(mesh, h, hu, hv, b, 0.0, dt), cfg, 4)
