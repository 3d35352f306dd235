"""The benchmark configurations at their stated sizes, on the GPU, bit for bit
against the oracle after every step.

Radial dam break: 2^16 cells (reference depth 15), uniform, 100 steps, f-wave,
Courant 0.5, reflecting (SLIP) walls and the OUTFLOW variant; compared with
the oracle's literal walk of the reference traversal (cell grammar reversed
every step) after each of the 100 steps, the run loop of src/SWE/SWE.f90:380-429
(one traversal per step, time and dt from the previous step).

Adaptive bowl: the a-priori mesh between depths 12 and 22, a remesh before
every step, 10 steps, each tree checked against the oracle's own adaption.
"""
import numpy as np
import pytest

from samoa_gb300 import scenarios

from .test_gpu_step import run_compare_walk

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("boundary", ["slip", "outflow"])
def test_dam_break_full_size_100_steps(swe_lib, oracle_lib, boundary):
    scn = scenarios.radial_dam_break(log2_cells=16, boundary=boundary)
    assert scn.grid.mesh.n_cells == 1 << 16 and scn.steps == 100
    run_compare_walk(scn, scn.steps)


def test_adaptive_bowl_full_size_remesh_every_step(swe_lib, oracle_lib):
    """Adaptive wet/dry bowl: depths 12..22 (the a-priori mesh is uniform at 22,
    2^23 cells), augmented Riemann solver, dry tolerance 1e-3, a remesh before
    every step (nadapt 1), 10 steps. The product remeshes on the host and the
    GPU steps on its trees; the oracle remeshes on its own (oracle_adapt with the
    integrated bowl bathymetry) and walks its own trees. After every step the
    state, flags, refinement count, time and dt agree bit for bit, and at every
    remesh the trees, transferred states and b."""
    from oracle import oracle as O

    from samoa_gb300 import swe

    from .helpers import assert_state_equal, oracle_params
    scn = scenarios.adaptive_bowl(min_depth=12, max_depth=22)
    g, cfg = scn.grid, scn.cfg
    assert cfg.flux_solver == "aug_riemann" and cfg.dry_tolerance == 1e-3
    assert g.mesh.n_cells == 1 << 23
    P = oracle_params(cfg)
    spec = O.bath_spec("bowl", 10.0, 0.4, cfg.scaling, cfg.offset, cfg.i_max_depth)
    mesh, h, hu, hv, b, t, dt = g.mesh, g.h, g.hu, g.hv, g.b, g.r_time, g.r_dt
    od, ost = mesh.depth.copy(), [h, hu, hv, O.bathymetry_cells(mesh.depth, spec)]
    assert np.array_equal(ost[3], b)
    ctx = swe.SweContext(0)
    sizes = []
    try:
        ctx.set_params(cfg.params())
        for k in range(10):
            if k > 0:
                flags, _ = ctx.refinements()
                gh, ghu, ghv, _ = ctx.download_state()
                t, dt, _ = ctx.get_time()
                mesh, (h, hu, hv, b) = swe.remesh(cfg, mesh, flags, gh, ghu, ghv, b, scenarios.bowl_bathymetry)
                od, _, ost = O.adapt(od, W.flags, W.h, W.hu, W.hv, W.b, spec=spec)
                assert np.array_equal(mesh.depth, od), "step %d: trees differ" % k
                for name, x, y in zip(("h", "hu", "hv", "b"), (h, hu, hv, b), ost):
                    assert np.array_equal(x, y), "step %d: transferred %s differs" % (k, name)
            W = O.WalkState(O.mesh_from_depths(od)["cells5"], *ost, t, dt)
            ctx.upload_mesh(mesh)
            ctx.upload_state(h, hu, hv, b)
            ctx.set_time(t, dt)
            W.steps(P, 1)
            ctx.traverse(1)
            gh, ghu, ghv, _ = ctx.download_state()
            assert_state_equal("step %d (%d cells)" % (k, mesh.n_cells), gh, ghu, ghv, W.h, W.hu, W.hv)
            flags, nref = ctx.refinements()
            assert np.array_equal(flags, W.flags) and nref == W.n_refine, "step %d" % k
            assert ctx.get_time() == (W.time, W.dt, W.dt_new), "step %d" % k
            sizes.append(mesh.n_cells)
    finally:
        ctx.close()
    assert sizes[-1] < sizes[0] // 4  # the flat water coarsened
