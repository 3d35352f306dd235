"""GPU discrete adjoint of the step (f-wave, augmented and Lax-Friedrichs
fluxes): one-step VJP against torch autograd of the FP64 restatement, the
checkpointed multi-step gauge gradient
against the FP64 CPU adjoint, and the gradient against central finite
differences (frozen dt sequence)."""
import ctypes as C

import numpy as np
import pytest

from oracle import swe_torch as ST
from samoa_gb300 import _lib, adjoint, scenarios, swe

from .helpers import random_states_scenario

pytestmark = pytest.mark.gpu


def _vp(t):
    return C.c_void_p(t.data_ptr())


def _prep(scn, warm_steps):
    """The scenario advanced a few steps on the CPU oracle so momenta are nonzero."""
    from .helpers import omp_state, oracle_params
    g = scn.grid
    S = omp_state(g.mesh, g)
    S.steps(oracle_params(scn.cfg), warm_steps)
    return S.h.copy(), S.hu.copy(), S.hv.copy(), g.b.copy(), float(S.scal[1])


CASES = [("bowl_outflow", "fwave"), ("bowl_noslip", "fwave"), ("dam_slip", "fwave"), ("dam_outflow", "fwave"),
         ("bowl_outflow", "llfbath"), ("bowl_noslip", "lfbath"), ("dam_slip", "lf"), ("dam_outflow", "llf"),
         ("bowl_outflow", "aug_riemann"), ("bowl_noslip", "aug_riemann"), ("dam_slip", "aug_riemann"),
         ("random", "aug_riemann"), ("random", "fwave"), ("random", "llfbath")]


@pytest.mark.parametrize("case,solver", CASES)
@pytest.mark.parametrize("parity", [0, 1])
def test_adjoint_step_matches_torch_vjp(swe_lib, case, solver, parity):
    import torch
    if case == "random":
        scn = random_states_scenario(solver)
    elif case.startswith("bowl"):
        scn = scenarios.parabolic_bowl(log2_cells=10, solver=solver, amplitude=2.5, sigma=0.08)
        scn.cfg.boundary = "noslip" if case.endswith("noslip") else "outflow"
    else:
        scn = scenarios.radial_dam_break(log2_cells=10, boundary=case.split("_")[1], solver=solver)
    if solver in ("lf", "llf"):  # the fluxes without bathymetry take the surface as the depth: b = 0, all wet
        g = scn.grid
        g.h[:] = (g.h - g.b) + 1.0
        g.b[:] = 0.0
        scn.cfg.courant_number = 0.05
        g.r_dt = swe.initial_dt(g.mesh, g.h, g.hu, g.hv, g.b, scn.cfg.courant_number)
    h, hu, hv, b, dt = _prep(scn, 6)
    mesh = scn.grid.mesh
    n = mesh.n_cells
    rng = np.random.default_rng(3 + parity)
    lam = rng.normal(size=(3, n))

    # torch reference VJP at the given parity
    T = ST.TorchStep(mesh, scaling=scn.cfg.scaling, drytol=scn.cfg.dry_tolerance, bc=scn.cfg.boundary,
                     solver=solver)
    x = [torch.tensor(a, requires_grad=True) for a in (h, hu, hv)]
    bb = torch.tensor(b, requires_grad=True)
    out = T.step(*x, bb, dt, parity)
    ref = torch.autograd.grad(out, x + [bb], grad_outputs=[torch.tensor(l) for l in lam], allow_unused=True)
    ref = [r.numpy() if r is not None else np.zeros(n) for r in ref]

    dev = torch.device("cuda", 0)
    ctx = swe.SweContext(0)
    try:
        ctx.set_params(scn.cfg.params())
        ctx.upload_mesh(mesh)
        ctx.upload_state(h, hu, hv, b)
        ctx.set_time(0.0, dt)
        ctx.set_dt_sequence(np.array([dt, dt]))
        if parity:  # bring the context to step 1 with the same state x
            ctx.traverse(1)
            ctx.synchronize()
            st = [torch.tensor(a, device=dev) for a in (h, hu, hv)]
            _lib.check(ctx.L.swe_snapshot_restore(ctx.ptr, _vp(st[0]), _vp(st[1]), _vp(st[2]), 1))
        lt = torch.tensor(lam, device=dev)
        o = torch.zeros_like(lt)
        gb = torch.zeros(n, dtype=torch.float64, device=dev)
        _lib.check(ctx.L.swe_adjoint_step(ctx.ptr, None, _vp(lt[0]), _vp(lt[1]), _vp(lt[2]), _vp(o[0]),
                                          _vp(o[1]), _vp(o[2]), _vp(gb)))
        ctx.synchronize()
        got = [o[0].cpu().numpy(), o[1].cpu().numpy(), o[2].cpu().numpy(), gb.cpu().numpy()]
    finally:
        ctx.close()
    for name, g_, r_ in zip(("h", "hu", "hv", "b"), got, ref):
        scale = max(np.abs(r_).max(), 1e-300)
        err = np.abs(g_ - r_).max() / scale
        assert err < 1e-11, (case, solver, parity, name, err)


@pytest.mark.parametrize("solver", ["fwave", "aug_riemann", "llfbath"])
def test_gauge_gradient_matches_cpu_adjoint(swe_lib, solver):
    """J over 40 steps with wet/dry fronts, 3 snapshot slots (forces recomputation):
    GPU checkpointed adjoint against torch autograd of the FP64 restatement."""
    import torch
    scn = scenarios.parabolic_bowl(log2_cells=10, solver=solver, amplitude=2.5, sigma=0.08)
    mesh, cfg = scn.grid.mesh, scn.cfg
    params = cfg.params()
    h0, b = scn.grid.h.copy(), scn.grid.b.copy()
    steps = 40
    dts = adjoint.record_dts(mesh, params, h0, b, steps)
    rng = np.random.default_rng(8)
    gauges = np.sort(rng.choice(np.nonzero(b < -3.0)[0], 12, replace=False))
    obs = rng.normal(0, 0.05, (steps, len(gauges)))
    P = adjoint.GaugeProblem(mesh, params, gauges, obs, dts, snapshots=3)
    try:
        J, gh, gbar = P.gradient(h0, b)
    finally:
        P.close()
    T = ST.TorchStep(mesh, scaling=cfg.scaling, drytol=cfg.dry_tolerance, bc=cfg.boundary, solver=solver)
    z = torch.zeros(mesh.n_cells, dtype=torch.float64)
    Jr, ghr, gbr = ST.gauge_objective_and_grad(T, torch.tensor(h0), z, z, torch.tensor(b), dts,
                                               torch.tensor(gauges), torch.tensor(obs))
    assert abs(J - Jr) <= 1e-12 * abs(Jr)
    for g_, r_ in ((gh.cpu().numpy(), ghr.numpy()), (gbar.cpu().numpy(), gbr.numpy())):
        err = np.abs(g_ - r_).max() / np.abs(r_).max()
        assert err < 1e-9, (solver, err)


def test_gradient_matches_central_differences_h0(swe_lib):
    """Deep basin, 200 steps, 6 seeded random directions of the initial
    displacement: central differences of J on the GPU (frozen dt sequence)
    agree with the adjoint gradient within 1e-6 relative. The step is 1e-5 of
    max|h0|: J carries ~1e-14 relative round-off, and at 1e-6 that is already
    1e-6 of the smaller directional derivatives (1e-2 of J)."""
    case = scenarios.adjoint_case(log2_cells=12, steps=200, n_gauges=16, seed=5)
    P = adjoint.GaugeProblem(case["mesh"], case["params"], case["gauges"], case["obs"], case["dts"], snapshots=8)
    try:
        J, gh, gb = P.gradient(case["h0"], case["b"])
        gh = gh.cpu().numpy()
        rng = np.random.default_rng(16)
        for k in range(6):
            d = rng.normal(size=case["h0"].shape)
            eps = 1e-5 * np.abs(case["h0"]).max()
            Jp = P.objective(case["h0"] + eps * d, case["b"], record=False)
            Jm = P.objective(case["h0"] - eps * d, case["b"], record=False)
            fd, ad = (Jp - Jm) / (2 * eps), float(gh @ d)
            assert abs(fd - ad) <= 1e-6 * abs(ad), (k, fd, ad)
    finally:
        P.close()


def _current_case(steps=100, n_gauges=12, seed=8):
    """The current basin with a frozen dt (0.8 of the CFL step of its first
    step, taken with the scaled geometry), seeded gauges and observations."""
    scn = scenarios.current_basin(log2_cells=12)
    g = scn.grid
    ctx = swe.SweContext(0)
    try:
        ctx.set_params(scn.cfg.params())
        ctx.upload_mesh(g.mesh)
        ctx.upload_state(g.h, g.hu, g.hv, g.b)
        ctx.set_time(0.0, g.r_dt)
        ctx.traverse(1)
        _, dt, _ = ctx.get_time()
    finally:
        ctx.close()
    rng = np.random.default_rng(seed)
    gauges = np.sort(rng.choice(g.mesh.n_cells, n_gauges, replace=False))
    obs = rng.normal(0.0, 0.05, (steps, n_gauges))
    return scn, np.full(steps, 0.8 * dt), gauges, obs


def test_gradient_plain_differences_under_a_current(swe_lib):
    """Moving water everywhere (a uniform current of (2, 1) m/s over a deep,
    rough basin, 100 steps): no wave speed sits at 0 and nothing is dry, so J
    has no jumps and plain central differences (no branch freezing) agree with
    the adjoint gradient within 1e-6 relative, in 6 seeded directions of the
    initial surface and 3 of the bathymetry (momenta held)."""
    scn, dts, gauges, obs = _current_case()
    g = scn.grid
    P = adjoint.GaugeProblem(g.mesh, scn.cfg.params(), gauges, obs, dts, snapshots=8)
    try:
        J, gh, gb = P.gradient_python(g.h, g.b, g.hu, g.hv)
        gh, gb = gh.cpu().numpy(), gb.cpu().numpy()
        assert abs(P.objective(g.h, g.b, record=False, hu0=g.hu, hv0=g.hv) - J) <= 1e-12 * abs(J)
        rng = np.random.default_rng(18)
        for key, grad, n_dir in (("h0", gh, 6), ("b", gb, 3)):
            for k in range(n_dir):
                d = rng.normal(size=g.mesh.n_cells)
                if key == "h0":
                    eps = 1e-5 * np.abs(g.h).max()
                    J_ = lambda s_: P.objective(g.h + s_ * eps * d, g.b, record=False, hu0=g.hu, hv0=g.hv)
                else:
                    eps = 1e-7 * np.abs(g.b).max()
                    J_ = lambda s_: P.objective(g.h, g.b + s_ * eps * d, record=False, hu0=g.hu, hv0=g.hv)
                fd, ad = (J_(1) - J_(-1)) / (2 * eps), float(grad @ d)
                assert abs(fd - ad) <= 1e-6 * abs(ad), (key, k, fd, ad)
    finally:
        P.close()


def test_bathymetry_gradient_matches_branch_frozen_differences(swe_lib):
    """The bathymetry gradient against central differences of the branch-frozen
    objective: J has kinks (the Einfeldt min/max and the middle wave's sign
    switch wherever neighbouring depths or velocities cross), so plain
    differences straddle them; replaying every branch of the unperturbed run
    (torch FP64 restatement) gives the function the adjoint differentiates.
    The step is 1e-4 of max|b|: the directional derivatives here are ~1e-6 of
    J, so smaller steps are limited by J's round-off; the frozen function is
    smooth, and the truncation error at this step is below 1e-7."""
    import torch
    case = scenarios.adjoint_case(log2_cells=10, steps=60, n_gauges=8, seed=7)
    P = adjoint.GaugeProblem(case["mesh"], case["params"], case["gauges"], case["obs"], case["dts"], snapshots=6)
    try:
        J, gh, gb = P.gradient(case["h0"], case["b"])
        gb = gb.cpu().numpy()
    finally:
        P.close()
    mesh, cfg = case["mesh"], case["cfg"]
    T = ST.TorchStep(mesh, scaling=cfg.scaling, drytol=cfg.dry_tolerance, bc=cfg.boundary)
    z = torch.zeros(mesh.n_cells, dtype=torch.float64)
    h0, b = torch.tensor(case["h0"]), torch.tensor(case["b"])
    g, obs = torch.tensor(case["gauges"]), torch.tensor(case["obs"])
    tapes = [ST.BranchTape() for _ in case["dts"]]
    J0 = ST.gauge_objective_frozen(T, h0, z, z, b, case["dts"], g, obs, tapes, False)
    assert abs(J0 - J) <= 1e-12 * abs(J)
    rng = np.random.default_rng(17)
    eps = 1e-4 * float(np.abs(case["b"]).max())
    for k in range(4):
        d = rng.normal(size=mesh.n_cells)
        dt_ = torch.tensor(d)
        Jp = ST.gauge_objective_frozen(T, h0, z, z, b + eps * dt_, case["dts"], g, obs, tapes, True)
        Jm = ST.gauge_objective_frozen(T, h0, z, z, b - eps * dt_, case["dts"], g, obs, tapes, True)
        fd, ad = (Jp - Jm) / (2 * eps), float(gb @ d)
        assert abs(fd - ad) <= 1e-6 * abs(ad), (k, fd, ad)


def test_autograd_function(swe_lib):
    """GaugeMisfit: forward is one forward run (T forward steps, no reverse
    step), backward the checkpointed sweep; J and the gradients are those of
    the problem's own objective and gradient."""
    import torch
    case = scenarios.adjoint_case(log2_cells=10, steps=30, n_gauges=8, seed=6)
    P = adjoint.GaugeProblem(case["mesh"], case["params"], case["gauges"], case["obs"], case["dts"], snapshots=4)
    try:
        h0 = torch.tensor(case["h0"], device="cuda", requires_grad=True)
        b = torch.tensor(case["b"], device="cuda", requires_grad=True)
        P.stats = {"forward_steps": 0, "adjoint_steps": 0}
        J = adjoint.GaugeMisfit.apply(h0, b, P)
        assert P.stats == {"forward_steps": 30, "adjoint_steps": 0}
        assert float(J.detach()) == P.objective(case["h0"], case["b"])
        P.stats = {"forward_steps": 0, "adjoint_steps": 0}
        J.backward()
        assert P.stats["adjoint_steps"] == 30 and P.stats["forward_steps"] >= 30
        J2, gh, gb = P.gradient(case["h0"], case["b"])
        assert abs(float(J.detach()) - J2) <= 1e-12 * abs(J2)
        assert torch.equal(h0.grad, gh) and torch.equal(b.grad, gb)
        with torch.no_grad():  # no gradient asked for: one forward run only
            P.stats = {"forward_steps": 0, "adjoint_steps": 0}
            adjoint.GaugeMisfit.apply(h0, b, P)
            assert P.stats == {"forward_steps": 30, "adjoint_steps": 0}
    finally:
        P.close()


def test_native_sweep_matches_python_sweep(swe_lib):
    """swe_gauge_gradient (the checkpointed sweep inside the library) against the
    same schedule driven step by step from Python: identical gradients, gauge
    series and forward-step counts; J up to its summation order."""
    import torch
    case = scenarios.adjoint_case(log2_cells=12, steps=150, n_gauges=16, seed=9)
    P = adjoint.GaugeProblem(case["mesh"], case["params"], case["gauges"], case["obs"], case["dts"], snapshots=5)
    try:
        P.stats = {"forward_steps": 0, "adjoint_steps": 0}
        J1, gh1, gb1 = P.gradient(case["h0"], case["b"])
        gv1 = P.gauge_values.clone()
        f1 = P.stats["forward_steps"]
        P.stats = {"forward_steps": 0, "adjoint_steps": 0}
        J2, gh2, gb2 = P.gradient_python(case["h0"], case["b"])
        f2 = P.stats["forward_steps"]
        assert torch.equal(gh1, gh2) and torch.equal(gb1, gb2)
        assert torch.equal(gv1, P.gauge_values)
        assert f1 == f2
        assert abs(J1 - J2) <= 1e-13 * abs(J2)
    finally:
        P.close()


def test_traverse_gauges_matches_step_by_step(swe_lib):
    import torch
    scn = scenarios.radial_dam_break(log2_cells=12, boundary="slip")
    g = scn.grid
    cells = torch.tensor([0, 17, 1000, g.mesh.n_cells - 1], dtype=torch.int64, device="cuda")
    dt0 = swe.initial_dt(g.mesh, g.h, g.hu, g.hv, g.b, scn.cfg.courant_number)
    out = []
    for batched in (True, False):
        ctx = swe.SweContext(0)
        try:
            ctx.set_params(scn.cfg.params())
            ctx.upload_mesh(g.mesh)
            ctx.upload_state(g.h, g.hu, g.hv, g.b)
            ctx.set_time(0.0, dt0)
            v = torch.empty((7, 4), dtype=torch.float64, device="cuda")
            if batched:
                _lib.check(ctx.L.swe_traverse_gauges(ctx.ptr, 7, 4, _vp(cells), _vp(v)))
            else:
                for k in range(7):
                    ctx.traverse(1)
                    _lib.check(ctx.L.swe_sample_gauges(ctx.ptr, 4, _vp(cells), _vp(v[k])))
            ctx.synchronize()
            out.append(v.cpu())
        finally:
            ctx.close()
    assert torch.equal(out[0], out[1])


def _windowed_case(solver="fwave"):
    """The wet/dry bowl on a 1024-cell mesh, refinement between depths 7 and 11,
    three windows of 8 steps with a remesh after each, 6 gauge points, a frozen dt
    small enough for the finest cells."""
    scn = scenarios.parabolic_bowl(log2_cells=10, solver=solver, amplitude=2.5, sigma=0.08, min_depth=7,
                                   max_depth=11)
    g, cfg = scn.grid, scn.cfg
    steps, window = 24, 8
    dts = np.full(steps, 0.25 * g.r_dt)
    rng = np.random.default_rng(21)
    cells = rng.choice(np.nonzero(g.b < -3.0)[0], 6, replace=False)
    pts = cfg.scaling * g.mesh.centroids[cells] + np.asarray(cfg.offset)
    obs = rng.normal(0, 0.05, (steps, len(pts)))
    return g, cfg, pts, obs, dts, window


def _torch_windowed_J(P, cfg, h0, b0, solver):
    """J of the windowed problem in the FP64 torch restatement, replaying P's plan."""
    import torch
    x = (h0, torch.zeros_like(h0), torch.zeros_like(h0))
    b = b0
    J = torch.zeros((), dtype=torch.float64)
    wins = P._windows()
    for w, (t0, t1) in enumerate(wins):
        mesh = P.plan["meshes"][w]
        T = ST.TorchStep(mesh, scaling=cfg.scaling, drytol=cfg.dry_tolerance, bc=cfg.boundary, solver=solver)
        gi = torch.as_tensor(P.plan["gauges"][w])
        for t in range(t0, t1):
            x = T.step(*x, b, float(P.dts[t]), t - t0)
            J = J + ((x[0][gi] - torch.as_tensor(P.obs[t])) ** 2).sum()
        if w + 1 < len(wins):
            tr = P.plan["transfers"][w]
            src = torch.as_tensor(tr.src)
            nxt = torch.clamp(src + 1, max=tr.n_old - 1)
            m = torch.as_tensor(tr.merged)
            app = lambda q: torch.where(m, 0.5 * (q[src] + q[nxt]), q[src])
            x = tuple(app(q) for q in x)
            b = app(b)
    return J


@pytest.mark.parametrize("solver", ["fwave", "aug_riemann"])
def test_windowed_gradient_matches_cpu_adjoint(swe_lib, solver):
    """Three 8-step windows on adaptive meshes (remesh from the flags after each,
    order-0 transfer, gauges re-located): the GPU gradient chained through the
    transfers' adjoints against torch autograd of the FP64 restatement replaying
    the same meshes and transfers."""
    import torch
    g, cfg, pts, obs, dts, window = _windowed_case(solver)
    P = adjoint.WindowedGaugeProblem(g.mesh, cfg, pts, obs, dts, window=window, snapshots=3)
    J, gh, gb = P.gradient(g.h, g.b)
    sizes = P.stats["cells"]
    assert len(set(sizes)) > 1, sizes  # the mesh did adapt between windows
    h0 = torch.tensor(g.h, requires_grad=True)
    b0 = torch.tensor(g.b, requires_grad=True)
    Jr = _torch_windowed_J(P, cfg, h0, b0, solver)
    ghr, gbr = torch.autograd.grad(Jr, [h0, b0])
    assert abs(J - float(Jr.detach())) <= 1e-11 * abs(float(Jr.detach()))
    for name, a, r in (("h0", gh, ghr.numpy()), ("b", gb, gbr.numpy())):
        err = np.abs(a - r).max() / np.abs(r).max()
        assert err < 1e-9, (solver, name, err)


def test_windowed_gradient_matches_central_differences(swe_lib):
    """The windowed objective with the plan frozen, on the deep (always wet) basin
    with the mesh adapting between depths 9 and 13: central differences in
    seeded directions of h0 against the gradient within 1e-6."""
    scn = scenarios.ocean_basin(log2_cells=12, steps=60)
    g, cfg = scn.grid, scn.cfg
    d = int(g.mesh.depth[0])
    cfg.i_min_depth, cfg.i_max_depth = d - 2, d + 2
    steps, window = 60, 20
    dts = np.full(steps, 0.4 * g.r_dt)
    rng = np.random.default_rng(25)
    deep = g.b < -100.0
    cells = rng.choice(np.nonzero(deep)[0], 8, replace=False)
    pts = cfg.scaling * g.mesh.centroids[cells] + np.asarray(cfg.offset)
    obs = rng.normal(0, 0.05, (steps, len(pts)))
    P = adjoint.WindowedGaugeProblem(g.mesh, cfg, pts, obs, dts, window=window, snapshots=4)
    J, gh, gb = P.gradient(g.h, g.b)
    assert len(set(P.stats["cells"])) > 1, P.stats["cells"]
    for _ in range(4):
        dd = rng.normal(size=g.mesh.n_cells) * deep
        eps = 1e-5 * np.abs(g.h).max()
        fd = (P.objective(g.h + eps * dd, g.b) - P.objective(g.h - eps * dd, g.b)) / (2 * eps)
        ad = float(gh @ dd)
        assert abs(fd - ad) <= 1e-6 * abs(ad), (fd, ad)


def test_windowed_gradient_matches_frozen_differences(swe_lib):
    """The windowed problem on the wet/dry bowl (meshes adapting between depths 7
    and 11): J of branch-frozen runs (each window's decisions recorded, then
    replayed) equals the plain J bit for bit at the recorded point, and its
    4-point central differences agree with the gradient within 1e-6 in random
    directions of h0 and of b, where plain differences cross wet/dry kinks."""
    g, cfg, pts, obs, dts, window = _windowed_case("fwave")
    P = adjoint.WindowedGaugeProblem(g.mesh, cfg, pts, obs, dts, window=window, snapshots=3)
    J, gh, gb = P.gradient(g.h, g.b)
    assert len(set(P.stats["cells"])) > 1, P.stats["cells"]
    assert P.objective(g.h, g.b) == J
    assert abs(P.stats["J_sweep"] - J) <= 1e-12 * abs(J)
    assert P.objective_frozen(g.h, g.b, record=True) == J
    assert P.objective_frozen(g.h, g.b, record=False) == J
    rng = np.random.default_rng(31)
    wet = (g.h - g.b) > cfg.dry_tolerance
    for key, grad, scale in (("h0", gh, np.abs(g.h - g.b).max()), ("b", gb, np.abs(g.b).max())):
        for _ in range(3):
            d = rng.normal(size=g.mesh.n_cells) * wet
            eps = 1e-4 * scale
            if key == "h0":
                Jf = lambda s_: P.objective_frozen(g.h + s_ * eps * d, g.b, record=False)
            else:
                Jf = lambda s_: P.objective_frozen(g.h, g.b + s_ * eps * d, record=False)
            fd = (8.0 * (Jf(1) - Jf(-1)) - (Jf(2) - Jf(-2))) / (12.0 * eps)
            ad = float(grad @ d)
            assert abs(fd - ad) <= 1e-6 * max(abs(ad), 1e-3 * np.linalg.norm(grad) * np.linalg.norm(d)), \
                (key, fd, ad)


def test_branch_frozen_runs_and_differences(swe_lib):
    """A recorded branch-frozen run equals the plain run bit for bit, its replay
    equals the recording, and 4-point central differences of the replayed J
    (truncation O(eps^4); no kink is crossed) agree with the adjoint gradient
    within 1e-6 in directions of h0 and of b."""
    case = scenarios.adjoint_case(log2_cells=12, steps=200, n_gauges=16, seed=5)
    P = adjoint.GaugeProblem(case["mesh"], case["params"], case["gauges"], case["obs"], case["dts"], snapshots=16)
    try:
        J0 = P.objective(case["h0"], case["b"], record=False)
        Jrec = P.objective_frozen(case["h0"], case["b"], record=True)
        Jrep = P.objective_frozen(case["h0"], case["b"], record=False)
        assert J0 == Jrec == Jrep, (J0, Jrec, Jrep)
        _, gh, gb = P.gradient(case["h0"], case["b"])
        gh, gb = gh.cpu().numpy(), gb.cpu().numpy()
        rng = np.random.default_rng(31)
        # h0: seeded random directions, relative error. b: J is far less sensitive to
        # the bathymetry (a random direction moves J by ~1e-8 of its ~1e-13-noisy
        # value), so one direction along the b-gradient with the relative error and
        # seeded ones with the error against |grad_b J| |d|
        dirs = [("h0", rng.normal(size=len(gh)), "rel") for _ in range(3)]
        dirs += [("b", gb / np.linalg.norm(gb), "rel")] + [("b", rng.normal(size=len(gb)), "norm") for _ in range(2)]
        for key, d, kind in dirs:
            eps = 1e-4 * np.abs(case[key]).max() / np.abs(d).max()  # smooth J: round-off sets the step
            x = case[key]
            args = (lambda v: (v, case["b"])) if key == "h0" else (lambda v: (case["h0"], v))
            J = lambda k: P.objective_frozen(*args(x + k * eps * d), record=False)
            fd = (8.0 * (J(1) - J(-1)) - (J(2) - J(-2))) / (12.0 * eps)
            g = gh if key == "h0" else gb
            ad = float(g @ d)
            ref = abs(ad) if kind == "rel" else np.linalg.norm(g) * np.linalg.norm(d)
            assert abs(fd - ad) <= 1e-6 * ref, (key, kind, fd, ad)
    finally:
        P.close()
