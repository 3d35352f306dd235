"""GPU parity on adaptive (mixed-depth) meshes: the step against the oracle
walk over the same tree, and a run with host remeshes between steps (the
remesh handoff: step flags -> swe_mesh_adapt -> swe_mesh_build -> upload)."""
import numpy as np
import pytest

from oracle import oracle as O
from samoa_gb300 import scenarios, swe

from .helpers import assert_state_equal, oracle_params

pytestmark = pytest.mark.gpu


def _upload(ctx, scn, mesh, h, hu, hv, b, time, dt):
    ctx.set_params(scn.cfg.params())
    ctx.upload_mesh(mesh)
    ctx.upload_state(h, hu, hv, b)
    ctx.set_time(time, dt)


@pytest.mark.parametrize("solver", ["fwave", "aug_riemann", "llfbath"])
def test_adaptive_mesh_step_bitexact(swe_lib, oracle_lib, solver):
    scn = scenarios.adaptive_dam_break(min_depth=6, max_depth=12, solver=solver, boundary="slip")
    g = scn.grid
    assert len(np.unique(g.mesh.depth)) >= 5
    o = O.mesh_from_depths(g.mesh.depth)
    W = O.WalkState(o["cells5"], g.h, g.hu, g.hv, g.b, g.r_time, g.r_dt)
    P = oracle_params(scn.cfg)
    ctx = swe.SweContext(0)
    try:
        _upload(ctx, scn, g.mesh, g.h, g.hu, g.hv, g.b, g.r_time, g.r_dt)
        for k in range(12):
            W.steps(P, 1)
            ctx.traverse(1)
            h, hu, hv, _ = ctx.download_state()
            flags, nref = ctx.refinements()
            tag = "%s step %d" % (solver, k)
            assert_state_equal(tag, h, hu, hv, W.h, W.hu, W.hv)
            assert np.array_equal(flags, W.flags), tag
            assert nref == W.n_refine, tag
            t, dt, dt_new = ctx.get_time()
            assert (t, dt, dt_new) == (W.time, W.dt, W.dt_new), tag
    finally:
        ctx.close()


def bowl_spec(cfg):
    return O.bath_spec("bowl", 10.0, 0.4, cfg.scaling, cfg.offset, cfg.i_max_depth)


def test_remesh_cycles_bitexact(swe_lib, oracle_lib):
    """Five cycles of four steps, each followed by a remesh from the last
    step's flags: the product remeshes on the host (swe.remesh) and the GPU
    steps on its trees; the oracle remeshes on its own (oracle_adapt, with the
    integrated bathymetry for refined cells) and walks its own trees. Trees,
    transferred states and b agree at every remesh, and the GPU matches the
    oracle bit for bit after every step."""
    scn = scenarios.adaptive_bowl(min_depth=6, max_depth=11, solver="fwave")
    g = scn.grid
    cfg = scn.cfg
    P = oracle_params(cfg)
    spec = bowl_spec(cfg)
    mesh, h, hu, hv, b, t, dt = g.mesh, g.h, g.hu, g.hv, g.b, g.r_time, g.r_dt
    od, ost = mesh.depth.copy(), [h, hu, hv, O.bathymetry_cells(mesh.depth, spec)]
    assert np.array_equal(ost[3], b)
    ctx = swe.SweContext(0)
    sizes = []
    try:
        for cycle in range(5):
            o = O.mesh_from_depths(od)
            W = O.WalkState(o["cells5"], *ost, t, dt)
            _upload(ctx, scn, mesh, h, hu, hv, b, t, dt)
            for k in range(4):
                W.steps(P, 1)
                ctx.traverse(1)
                gh, ghu, ghv, _ = ctx.download_state()
                assert_state_equal("cycle %d step %d" % (cycle, k), gh, ghu, ghv, W.h, W.hu, W.hv)
            flags, _ = ctx.refinements()
            assert np.array_equal(flags, W.flags)
            t, dt, _ = ctx.get_time()
            assert (t, dt) == (W.time, W.dt)
            mesh, (h, hu, hv, b) = swe.remesh(cfg, mesh, flags, gh, ghu, ghv, b, scenarios.bowl_bathymetry)
            od, _, ost = O.adapt(od, W.flags, W.h, W.hu, W.hv, W.b, spec=spec)
            assert np.array_equal(mesh.depth, od), "cycle %d: trees differ" % cycle
            for name, x, y in zip(("h", "hu", "hv", "b"), (h, hu, hv, b), ost):
                assert np.array_equal(x, y), "cycle %d: transferred %s differs" % (cycle, name)
            sizes.append(mesh.n_cells)
    finally:
        ctx.close()
    assert len(set(sizes)) > 1  # the mesh did change


def test_run_adaptive_bowl(swe_lib):
    """The run loop with a remesh before every step on the wet/dry bowl: the
    mesh coarsens the flat water, and the water volume changes only through the
    wet/dry clamps and the re-sampled bathymetry of refined cells."""
    scn = scenarios.adaptive_bowl(min_depth=6, max_depth=10)
    g = scn.grid
    vol0 = np.sum(np.maximum(g.h - g.b, 0.0) * np.ldexp(1.0, -(g.mesh.depth.astype(int) + 1)))
    (mesh, h, hu, hv, b, t, dt), st = swe.run_adaptive(scn.cfg, g.mesh, g.h, g.hu, g.hv, g.b, g.r_dt, 8,
                                                       bathymetry=scenarios.bowl_bathymetry)
    assert st["steps"] == 8 and st["remeshes"] == 7
    assert mesh.n_cells < g.mesh.n_cells
    vol = np.sum(np.maximum(h - b, 0.0) * np.ldexp(1.0, -(mesh.depth.astype(int) + 1)))
    assert abs(vol - vol0) < 5e-2 * vol0  # merging a wet cell with a dry one loses its negative depth
    assert t > 0 and dt > 0
