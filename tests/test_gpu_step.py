"""GPU parity of the fused SWE step against the oracle, through the C ABI.

Bar: bit-exact state (h, hu, hv), refinement flags, refinement count, time and
dt after every step, for every solver and boundary condition, against the
sequential walk that follows the reference traversal (cell grammar reversed
every step). At sizes the walk cannot reach in seconds the OpenMP oracle
(checked against the walk bit for bit in test_oracle.py) is the reference.
"""
import numpy as np
import pytest

from oracle import oracle as O
from samoa_gb300 import scenarios, swe

from .helpers import assert_state_equal, omp_state, oracle_params, random_states_scenario, walk_state

pytestmark = pytest.mark.gpu


def run_compare_walk(scn, steps, tiling=None):
    g = scn.grid
    depth = int(g.mesh.depth[0])
    W = walk_state(depth, g)
    P = oracle_params(scn.cfg)
    trav = swe.SweEulerTimestepTraversal(scn.cfg)
    if tiling:
        trav.set_tiling(*tiling)
    try:
        for k in range(steps):
            W.steps(P, 1)
            trav.traverse(g)
            tag = "%s step %d" % (scn.name, k)
            assert_state_equal(tag, g.h, g.hu, g.hv, W.h, W.hu, W.hv)
            assert np.array_equal(g.refinement, W.flags), tag + ": refinement flags differ"
            assert g.i_refinements_issued == W.n_refine, tag
            assert g.r_time == W.time and g.r_dt == W.dt, (tag, g.r_time, W.time, g.r_dt, W.dt)
            assert g.r_dt_new == W.dt_new, tag
    finally:
        trav.close()


@pytest.mark.parametrize("boundary", ["slip", "outflow", "noslip"])
def test_dam_break_fwave_bitexact(swe_lib, oracle_lib, boundary):
    scn = scenarios.radial_dam_break(log2_cells=12, boundary=boundary)
    run_compare_walk(scn, 12)


@pytest.mark.parametrize("solver", ["aug_riemann", "fwave", "llfbath", "lfbath"])
def test_bowl_wet_dry_bitexact(swe_lib, oracle_lib, solver):
    scn = scenarios.parabolic_bowl(log2_cells=12, solver=solver, amplitude=2.0, sigma=0.08)
    run_compare_walk(scn, 15)


@pytest.mark.parametrize("solver", ["lf", "llf"])
def test_lf_flat_bitexact(swe_lib, oracle_lib, solver):
    # the LF fluxes without bathymetry assume b = 0 (src/SWE/SWE_euler_timestep.f90:423); the
    # global variant diffuses with a fixed alpha = 100 m/s, stable only at small Courant numbers
    scn = scenarios.radial_dam_break(log2_cells=10, boundary="outflow", solver=solver)
    scn.cfg.courant_number = 0.05
    g = scn.grid
    g.b[:] = 0.0
    g.h[:] = g.h + 10.0
    g.r_dt = swe.initial_dt(g.mesh, g.h, g.hu, g.hv, g.b, scn.cfg.courant_number)
    run_compare_walk(scn, 10)


def test_refinement_flags_bitexact(swe_lib, oracle_lib):
    # dmin < depth < dmax so both refine and coarsen flags occur
    scn = scenarios.radial_dam_break(log2_cells=12, boundary="slip")
    scn.cfg.i_min_depth = 5
    scn.cfg.i_max_depth = 13
    run_compare_walk(scn, 8)


@pytest.mark.parametrize("tiling", [(64, 64), (96, 128), (1536, 256), (1024, 256), (256, 96), (64, 64, 2),
                                    (512, 128, 2), (1280, 256, 2)])
def test_tilings_bitexact(swe_lib, oracle_lib, tiling):
    """Segment length, block size and staging depth change nothing in the results."""
    scn = scenarios.parabolic_bowl(log2_cells=13, amplitude=1.0)
    run_compare_walk(scn, 6, tiling=tiling)


def test_dt_clamps(swe_lib, oracle_lib):
    scn = scenarios.radial_dam_break(log2_cells=10)
    scn.cfg.r_max_time = 1e-4
    scn.cfg.r_output_time_step = 5e-5
    run_compare_walk(scn, 5)


def test_large_mesh_against_omp(swe_lib, oracle_lib):
    scn = scenarios.ocean_basin(log2_cells=20, steps=6)
    g = scn.grid
    S = omp_state(g.mesh, g)
    P = oracle_params(scn.cfg)
    trav = swe.SweEulerTimestepTraversal(scn.cfg)
    try:
        for k in range(4):
            S.steps(P, 1)
            trav.traverse(g)
            assert_state_equal("basin step %d" % k, g.h, g.hu, g.hv, S.h, S.hu, S.hv)
            assert g.r_dt == S.scal[1] and g.r_time == S.scal[0]
    finally:
        trav.close()


@pytest.mark.parametrize("order", ["curve", "spread", "auto"])
@pytest.mark.parametrize("mode", ["pass", "inkernel"])
def test_cross_segment_modes_against_omp(swe_lib, oracle_lib, mode, order):
    """Edges between two segments solved once by the pass before the step kernel,
    or by both segments' CTAs, with segments handed out along the curve or
    spread: the same bits (state, flags, dt) as the oracle."""
    scn = scenarios.ocean_basin(log2_cells=16, steps=4)
    g = scn.grid
    S = omp_state(g.mesh, g)
    P = oracle_params(scn.cfg)
    trav = swe.SweEulerTimestepTraversal(scn.cfg)
    trav.set_tiling(256, 128)
    trav.ctx.set_cross_pass(mode)
    trav.ctx.set_segment_order(order)
    try:
        for k in range(4):
            S.steps(P, 1)
            trav.traverse(g)
            assert_state_equal("%s step %d" % (mode, k), g.h, g.hu, g.hv, S.h, S.hu, S.hv)
            assert np.array_equal(g.refinement, S.flags)
            assert g.r_dt == S.scal[1] and g.r_time == S.scal[0]
        counts = trav.ctx.task_counts()
        assert counts["segments"] == g.mesh.n_cells // 256 and counts["cross_edges"] > 0
        assert counts["launches_per_step"] == (2 if mode == "pass" else 1)
    finally:
        trav.close()


def _odd_mesh(depth):
    """A uniform mesh with its last cell removed: odd cell count, the removed
    cell's neighbours get boundary edges instead. Exercises ragged segments."""
    m = swe.uniform_mesh(depth)
    n = m.n_cells - 1
    keep = (m.edge_cells[:, 0] < n) & (m.edge_cells[:, 1] < n)
    ec, el = m.edge_cells[keep], m.edge_local[keep]
    cut = ~keep
    nb_c = np.where(m.edge_cells[cut, 0] < n, m.edge_cells[cut, 0], m.edge_cells[cut, 1])
    nb_l = np.where(m.edge_cells[cut, 0] < n, m.edge_local[cut, 0], m.edge_local[cut, 1])
    bk = m.bnd_cell < n
    bc = np.concatenate([m.bnd_cell[bk], nb_c])
    bl = np.concatenate([m.bnd_local[bk], nb_l]).astype(np.int8)
    return swe.Mesh(m.depth[:n].copy(), m.plotter[:n].copy(), ec.copy(), el.copy(), bc, bl, m.centroids[:n].copy())


def test_full_size_basin_against_omp(swe_lib, oracle_lib):
    """The bench workload itself, 2^26 cells with the autotuned tiling (384 x 128)
    and the cross-edge pass: 20 steps bit-exact against the OpenMP oracle, state,
    flags and dt compared after steps 1, 2, 3, 10 and 20 (time and dt carry every
    step's CFL maximum, so a step in between that differed would show)."""
    scn = scenarios.ocean_basin(log2_cells=26, steps=20, device="cuda")
    g = scn.grid
    S = omp_state(g.mesh, g)
    P = oracle_params(scn.cfg)
    trav = swe.SweEulerTimestepTraversal(scn.cfg)
    trav.set_tiling(384, 128)
    try:
        done = 0
        for k in (1, 1, 1, 7, 10):
            S.steps(P, k)
            trav.traverse(g, steps=k)
            done += k
            assert_state_equal("2^26 basin after %d steps" % done, g.h, g.hu, g.hv, S.h, S.hu, S.hv)
            assert np.array_equal(g.refinement, S.flags)
            assert g.r_dt == S.scal[1] and g.r_time == S.scal[0]
            assert g.r_dt_new == S.dt_new
    finally:
        trav.close()


@pytest.mark.parametrize("tiling", [(64, 64), (512, 256), (64, 64, 2)])
def test_odd_cell_count_against_omp(swe_lib, oracle_lib, tiling):
    mesh = _odd_mesh(9)
    assert mesh.n_cells % 2 == 1
    scn = scenarios.radial_dam_break(log2_cells=10, mesh=None)
    n = mesh.n_cells
    g = swe.Grid(mesh, scn.grid.h[:n].copy(), scn.grid.hu[:n].copy(), scn.grid.hv[:n].copy(), scn.grid.b[:n].copy(),
                 0.0, scn.grid.r_dt)
    S = omp_state(mesh, g)
    P = oracle_params(scn.cfg)
    trav = swe.SweEulerTimestepTraversal(scn.cfg)
    trav.set_tiling(*tiling)
    try:
        for k in range(6):
            S.steps(P, 1)
            trav.traverse(g)
            assert_state_equal("odd mesh step %d" % k, g.h, g.hu, g.hv, S.h, S.hu, S.hv)
            assert np.array_equal(g.refinement, S.flags)
    finally:
        trav.close()


def test_lake_at_rest_is_exact(swe_lib):
    scn = scenarios.lake_at_rest(log2_cells=12)
    g = scn.grid
    h0 = g.h.copy()
    trav = swe.SweEulerTimestepTraversal(scn.cfg)
    try:
        trav.traverse(g, steps=20)
        assert np.array_equal(g.h, h0)
        assert not g.hu.any() and not g.hv.any()
    finally:
        trav.close()


@pytest.mark.parametrize("boundary", ["outflow", "slip", "noslip"])
def test_rest_edges_bitexact(swe_lib, oracle_lib, boundary):
    """The f-wave step's lake-at-rest path (both sides wet, every momentum +-0,
    ((bR + dR) - bL) - dL a zero) against the oracle walk: a lake at rest over
    rough bathymetry where a quarter of the cells hold -0 momenta, some
    surfaces are one ulp off (their edges take the full path), some cells are
    dry land and one patch moves, so rest edges border moving and dry ones."""
    scn = scenarios.lake_at_rest(log2_cells=12)
    scn.cfg.boundary = boundary
    g = scn.grid
    n = g.mesh.n_cells
    rng = np.random.default_rng(42)
    neg = rng.random(n) < 0.25
    g.hu[neg] = -0.0
    g.hv[rng.random(n) < 0.25] = -0.0
    ulp = rng.random(n) < 0.05
    g.h[ulp] = np.nextafter(g.h[ulp], 1.0)
    dry = rng.random(n) < 0.03
    g.b[dry] = 0.5
    g.h[dry] = 0.0  # surface min(b, 0) on dry land
    patch = np.arange(n // 3, n // 3 + 64)
    g.hu[patch] = 0.3
    g.hv[patch] = -0.2
    g.r_dt = swe.initial_dt(g.mesh, g.h, g.hu, g.hv, g.b, scn.cfg.courant_number)
    run_compare_walk(scn, 12)


@pytest.mark.parametrize("solver", ["fwave", "aug_riemann", "llfbath"])
def test_all_dry_domain(swe_lib, oracle_lib, solver):
    """Dry land everywhere (surface at min(b, 0) below a positive bottom): no edge
    carries a flux, the state stays as it is, every flag is bit-exact with the
    oracle walk and dt_new stays at its initial huge value.

    dt is clamped by r_max_time (pre_traversal_grid_op,
    src/SWE/SWE_euler_timestep.f90:93-95): without it the step after the first
    runs with dt = courant * huge, -dt / volume overflows to -inf and the zero
    updates turn into NaN, in the reference as here."""
    d = 9
    mesh = swe.uniform_mesh(d)
    cfg = swe.Config(flux_solver=solver, boundary="outflow", courant_number=0.45, dry_tolerance=0.01,
                     scaling=1.0, offset=(-0.5, -0.5), i_min_depth=d, i_max_depth=d + 1, r_max_time=1.0)
    rng = np.random.default_rng(31)
    b = 1.0 + rng.random(mesh.n_cells)
    h = np.minimum(b, 0.0)
    g = swe.Grid(mesh, h.copy(), np.zeros(mesh.n_cells), np.zeros(mesh.n_cells), b, 0.0, 1e-3)
    scn = scenarios.Scenario("all_dry", g, cfg, 3)
    run_compare_walk(scn, 3)
    assert np.array_equal(g.h, h) and not g.hu.any() and not g.hv.any()
    assert g.r_dt_new == np.finfo(np.float64).max


def test_mass_conservation_and_drift(swe_lib, oracle_lib):
    """Mass is conserved to round-off (reflective walls, no wet/dry clamps);
    after 1,000 steps the GPU state still equals the oracle's bit for bit."""
    scn = scenarios.radial_dam_break(log2_cells=12, boundary="noslip")
    g = scn.grid
    vol = O.cell_volume(int(g.mesh.depth[0]))
    m0 = float(np.sum(g.h - g.b)) * vol
    S = omp_state(g.mesh, g)
    P = oracle_params(scn.cfg)
    trav = swe.SweEulerTimestepTraversal(scn.cfg)
    try:
        trav.traverse(g, steps=1000)
        S.steps(P, 1000)
        assert_state_equal("after 1000 steps", g.h, g.hu, g.hv, S.h, S.hu, S.hv)
        m1 = float(np.sum(g.h - g.b)) * vol
        # noslip ghost mirrors the momentum, so the boundary mass flux is round-off only
        assert abs(m1 - m0) / m0 < 1e-11, (m0, m1)
    finally:
        trav.close()


@pytest.mark.parametrize("huge", [False, True])
@pytest.mark.parametrize("tiling", [(64, 64), (384, 128)])
def test_cfl_bound_near_ties(swe_lib, oracle_lib, tiling, huge):
    """The cell update skips a cell's CFL speed sum when a float upper bound of
    its key stays below the largest key its warp has taken (key_below): dt_new
    must still be the maximum over every cell, bit for bit with the oracle.
    A lake at rest over random depths 10..15 m (so most cells are skipped once
    a warp has met a deep one), whose deepest depth recurs at scattered cells
    and, 2e-12 relative deeper (far inside the bound's 2^-20 margin), at one
    cell near the end of the curve; with `huge`, one cell 1e60 m deep, whose
    speed (~3e30) lies outside the range the bound handles. 2^18 cells in
    64- or 384-cell segments: several segments per CTA, so warps carry a
    running maximum from segment to segment."""
    d = 18
    mesh = swe.uniform_mesh(d)
    n = mesh.n_cells
    rng = np.random.default_rng(77)
    b = -(10.0 + 5.0 * rng.random(n))
    m = int(np.argmin(b))
    ties = rng.choice(n, 64, replace=False)
    b[ties] = b[m]
    b[n - 1 - int(rng.integers(0, 1000))] = b[m] * (1.0 + 2e-12)
    if huge:
        b[int(rng.integers(n // 2, n))] = -1e60
    h = np.zeros(n)
    cfg = swe.Config(flux_solver="fwave", boundary="outflow", courant_number=0.45, dry_tolerance=1e-3,
                     scaling=1.0, offset=(-0.5, -0.5), i_min_depth=d - 1, i_max_depth=d + 1)
    g = swe.Grid(mesh, h, np.zeros(n), np.zeros(n), b, 0.0, 1e-6)
    S = omp_state(mesh, g)
    P = oracle_params(cfg)
    trav = swe.SweEulerTimestepTraversal(cfg)
    trav.set_tiling(*tiling)
    try:
        for k in range(3):
            trav.traverse(g)
            S.steps(P, 1)
            tag = "near ties %s step %d" % (tiling, k)
            assert_state_equal(tag, g.h, g.hu, g.hv, S.h, S.hu, S.hv)
            assert g.r_dt_new == S.dt_new, (tag, g.r_dt_new, S.dt_new)
            assert g.r_time == S.scal[0] and g.r_dt == S.scal[1], tag
    finally:
        trav.close()


def test_determinism(swe_lib):
    out = []
    for _ in range(2):
        scn = scenarios.parabolic_bowl(log2_cells=14, amplitude=1.0)
        trav = swe.SweEulerTimestepTraversal(scn.cfg)
        trav.traverse(scn.grid, steps=25)
        trav.close()
        out.append(np.concatenate([scn.grid.h, scn.grid.hu, scn.grid.hv]).view(np.uint64))
    assert np.array_equal(out[0], out[1])


def test_riemann_batch_against_oracle(swe_lib, oracle_lib):
    """Solver-level check on targeted edge states: wet/wet, dry/dry, wet/dry,
    walls, supercritical flow, transcritical, random normals."""
    import ctypes as C
    from samoa_gb300 import _lib
    rng = np.random.default_rng(11)
    n = 20000
    normals = rng.normal(size=(n, 2))
    normals /= np.linalg.norm(normals, axis=1, keepdims=True)
    bl = rng.uniform(-20, 5, n)
    br = bl + rng.choice([0.0, 1.0], n) * rng.uniform(-10, 10, n)
    dl = rng.choice([0.0, 1e-4, 1.0], n, p=[0.2, 0.1, 0.7]) * rng.uniform(0, 20, n)
    dr = rng.choice([0.0, 1e-4, 1.0], n, p=[0.2, 0.1, 0.7]) * rng.uniform(0, 20, n)
    ql = np.stack([bl + dl, rng.normal(0, 30, n), rng.normal(0, 30, n), bl], 1)
    qr = np.stack([br + dr, rng.normal(0, 30, n), rng.normal(0, 30, n), br], 1)
    # degenerate families: water at rest (zero momenta), equal depths, identical
    # states, slow flow over equal bottoms (zero and near-zero Cramer numerators,
    # sonic tests on both sides of their thresholds)
    m = n // 5
    k = np.arange(n)
    rest = k % 5 == 0
    ql[rest, 1:3] = 0.0
    qr[rest, 1:3] = 0.0
    eqd = k % 5 == 1
    qr[eqd, 0] = qr[eqd, 3] + (ql[eqd, 0] - ql[eqd, 3])
    same = k % 5 == 2
    qr[same] = ql[same]
    slow = k % 5 == 3
    qr[slow, 3] = ql[slow, 3]
    ql[slow, 1:3] = rng.normal(0, 1e-7, (int(slow.sum()), 2))
    qr[slow, 1:3] = rng.normal(0, 1e-7, (int(slow.sum()), 2))
    assert m > 0
    drytol = 1e-3
    L = _lib.load()
    for solver in (swe.FWAVE, swe.AUG_RIEMANN, swe.LF_BATH, swe.LLF_BATH):
        gl, gr = np.zeros((n, 4)), np.zeros((n, 4))
        p = lambda a: np.ascontiguousarray(a).ctypes.data_as(C.c_void_p)
        _lib.check(L.swe_riemann_batch(solver, n, p(normals), p(ql), p(qr), drytol, p(gl), p(gr)))
        ol, orr = np.zeros((n, 4)), np.zeros((n, 4))
        for i in range(n):
            ol[i], orr[i] = O.edge_flux(solver, normals[i], ql[i], qr[i], drytol)
        ok = np.isfinite(ol).all(1) & np.isfinite(orr).all(1)
        assert np.array_equal(gl[ok], ol[ok]) and np.array_equal(gr[ok], orr[ok]), solver
        assert np.array_equal(np.isfinite(gl).all(1) & np.isfinite(gr).all(1), ok), solver


@pytest.mark.parametrize("depth", [0, 1, 2, 4])
@pytest.mark.parametrize("solver", ["fwave", "aug_riemann", "llfbath"])
def test_tiny_meshes_bitexact(swe_lib, oracle_lib, depth, solver):
    """Meshes of 2 to 32 cells (one segment, no edges between segments, most
    cells on the boundary): random wet/dry states, bit for bit against the walk."""
    scn = random_states_scenario(solver, seed=7 + depth, depth=depth)
    run_compare_walk(scn, 6)


def test_contexts_with_different_tilings_interleave(swe_lib, oracle_lib):
    """Two contexts of one process with different segment lengths, stepped in
    turns (a kernel's shared-memory limit is an attribute of the function, not
    of a context): both run and match the oracle bit for bit."""
    scns = [scenarios.radial_dam_break(log2_cells=12, boundary="slip"),
            scenarios.parabolic_bowl(log2_cells=12, solver="fwave", amplitude=2.0, sigma=0.08)]
    travs = [swe.SweEulerTimestepTraversal(s.cfg) for s in scns]
    try:
        travs[0].set_tiling(1024, 256)
        travs[1].set_tiling(128, 128)
        refs = [(omp_state(s.grid.mesh, s.grid), oracle_params(s.cfg)) for s in scns]
        for k in range(3):
            for s, t, (S, P) in zip(scns, travs, refs):
                S.steps(P, 1)
                t.traverse(s.grid)
                assert_state_equal("%s step %d" % (s.name, k), s.grid.h, s.grid.hu, s.grid.hv, S.h, S.hu, S.hv)
    finally:
        for t in travs:
            t.close()


def test_tiling_limits(swe_lib):
    scn = scenarios.radial_dam_break(log2_cells=8)
    trav = swe.SweEulerTimestepTraversal(scn.cfg)
    try:
        with pytest.raises(swe._lib.SweError):
            trav.set_tiling(2048, 256)
        with pytest.raises(swe._lib.SweError):
            trav.set_tiling(512, 100)
        trav.set_tiling(128, 128)
        trav.traverse(scn.grid)
    finally:
        trav.close()


@pytest.mark.parametrize("solver", ["fwave", "aug_riemann"])
def test_fma_mode_within_tolerance(swe_lib, oracle_lib, solver):
    """FMA arithmetic: each step from the oracle's state agrees within 1e-12
    (max-norm, relative to the field's max) and the flags are equal; the drift
    after 100 steps is stated, not hidden."""
    scn = scenarios.parabolic_bowl(log2_cells=12, solver=solver, amplitude=2.0, sigma=0.08, min_depth=6,
                                   max_depth=13)
    g = scn.grid
    S = omp_state(g.mesh, g)
    P = oracle_params(scn.cfg)
    ctx = swe.SweContext(0)
    try:
        ctx.set_params(scn.cfg.params())
        ctx.set_arith("fma")
        ctx.upload_mesh(g.mesh)
        for k in range(5):  # one FMA step from the oracle's exact state, each time
            ctx.upload_state(S.h, S.hu, S.hv, g.b)
            ctx.set_time(S.scal[0], S.scal[1])
            import ctypes as C
            S.steps(P, 1)
            ctx.traverse(1)
            h, hu, hv, _ = ctx.download_state()
            for a, r in ((h, S.h), (hu, S.hu), (hv, S.hv)):
                assert np.abs(a - r).max() <= 1e-12 * np.abs(r).max()
            flags, _ = ctx.refinements()
            assert np.array_equal(flags, S.flags)
    finally:
        ctx.close()


@pytest.mark.parametrize("span", [30, 500, 1022])
def test_division_with_shared_reciprocal_is_ieee(swe_lib, span):
    """The step's quotients by a shared reciprocal (Markstein's correction) equal
    IEEE division bit for bit: 2 x 2^24 seeded pairs per exponent span, the
    widest one reaching the ranges where plain division takes over."""
    import ctypes as C
    from samoa_gb300 import _lib
    bad = C.c_int64(-1)
    _lib.check(swe_lib.swe_division_check(1 << 24, 1234 + span, span, C.byref(bad)))
    assert bad.value == 0


