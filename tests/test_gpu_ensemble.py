"""GPU ensembles: many instances in one launch per step, each bit-identical to
its own plain run; CUDA-graph replay identical to plain launches; frozen dt
sequences."""
import numpy as np
import pytest

from samoa_gb300 import scenarios, swe

from .helpers import assert_state_equal, omp_state, oracle_params, random_states_scenario
from .test_gpu_step import _odd_mesh

pytestmark = pytest.mark.gpu


def _tiny_members():
    """Instances of 2, 4 and 32 cells (random wet/dry states, f-wave)."""
    out = []
    for depth in (0, 1, 4):
        scn = random_states_scenario("fwave", seed=11 + depth, depth=depth)
        out.append((scn.grid.mesh, scn.grid, scn.cfg))
    return out


def _ensemble_members(tiny=False):
    members = []
    ens = scenarios.bowl_ensemble(n_instances=5, seed=9, log2_range=(8, 13))
    for m, g, c in zip(ens.meshes, ens.grids, ens.cfgs):
        members.append((m, g, c))
    # an odd-sized instance with another boundary condition and dry tolerance
    odd = _odd_mesh(7)
    base = scenarios.radial_dam_break(log2_cells=8, boundary="slip")
    n = odd.n_cells
    g = swe.Grid(odd, base.grid.h[:n].copy(), base.grid.hu[:n].copy(), base.grid.hv[:n].copy(),
                 base.grid.b[:n].copy(), 0.0, base.grid.r_dt)
    cfg = base.cfg
    cfg.i_min_depth, cfg.i_max_depth = 3, 9
    members.insert(2, (odd, g, cfg))
    if tiny:  # first, in the middle and last
        t = _tiny_members()
        members = [t[0]] + members[:3] + [t[1]] + members[3:] + [t[2]]
    return members


def _upload(ens, members):
    ens.upload_meshes([m for m, _, _ in members])
    ens.set_params_list([c.params() for _, _, c in members])
    cat = lambda k: np.concatenate([getattr(g, k) for _, g, _ in members])
    ens.upload_state(cat("h"), cat("hu"), cat("hv"), cat("b"))
    ens.set_times([g.r_time for _, g, _ in members], [g.r_dt for _, g, _ in members])


@pytest.mark.parametrize("graph,staging,tiny", [(False, 1, False), (True, 1, False), (False, 2, False),
                                               (True, 1, True)])
def test_ensemble_members_match_oracle(swe_lib, oracle_lib, graph, staging, tiny):
    members = _ensemble_members(tiny)
    ens = swe.SweEnsemble(0)
    try:
        ens.set_tiling(128, 128)
        ens.set_staging(staging)
        _upload(ens, members)
        refs = [omp_state(m, g) for m, g, _ in members]
        steps = 7
        for S, (_, _, c) in zip(refs, members):
            S.steps(oracle_params(c), steps)
        if graph:
            ens.traverse_graph(steps)
        else:
            ens.traverse(steps)
        ens.synchronize()
        h, hu, hv, _ = ens.download_state()
        flags, nref = ens.refinements_all()
        t, dt, _ = ens.get_times()
        for i, (S, hh, uu, vv, ff) in enumerate(zip(refs, ens.split(h), ens.split(hu), ens.split(hv),
                                                    ens.split(flags))):
            assert_state_equal("instance %d" % i, hh, uu, vv, S.h, S.hu, S.hv)
            assert np.array_equal(ff, S.flags)
            assert nref[i] == S.n_refine
            assert t[i] == S.scal[0] and dt[i] == S.scal[1]
    finally:
        ens.close()


def test_graph_replay_equals_launches(swe_lib):
    out = []
    for graph in (False, True):
        scn = scenarios.parabolic_bowl(log2_cells=14, amplitude=2.0)
        ctx = swe.SweContext(0)
        ctx.set_params(scn.cfg.params())
        ctx.upload_mesh(scn.grid.mesh)
        ctx.upload_state(scn.grid.h, scn.grid.hu, scn.grid.hv, scn.grid.b)
        ctx.set_time(0.0, scn.grid.r_dt)
        for _ in range(3):
            if graph:
                ctx.traverse_graph(4)
            else:
                ctx.traverse(4)
        ctx.synchronize()
        out.append((np.concatenate(ctx.download_state()[:3]), ctx.get_time(), ctx.step_count()))
        ctx.close()
    assert np.array_equal(out[0][0], out[1][0]) and out[0][1] == out[1][1] and out[0][2] == out[1][2] == 12


def test_frozen_dt_sequence(swe_lib, oracle_lib):
    """With a frozen dt sequence the step uses exactly those dts (CFL dt ignored)."""
    scn = scenarios.radial_dam_break(log2_cells=10)
    g = scn.grid
    ctx = swe.SweContext(0)
    try:
        ctx.set_params(scn.cfg.params())
        ctx.upload_mesh(g.mesh)
        ctx.upload_state(g.h, g.hu, g.hv, g.b)
        ctx.set_time(0.0, g.r_dt)
        dts = np.array([1e-4, 2e-4, 5e-5])
        ctx.set_dt_sequence(dts)
        ctx.traverse(3)
        t, _, _ = ctx.get_time()
        assert t == (1e-4 + 2e-4) + 5e-5
        h = ctx.download_state()[0]
        S = omp_state(g.mesh, g)
        P = oracle_params(scn.cfg)
        for d in dts:
            S.scal[1] = d
            S.steps(P, 1)
        assert np.array_equal(h, S.h)
    finally:
        ctx.close()
