"""Synthetic SWE scenarios on uniform Sierpinski meshes (host-side setup).

The reference hard-codes a 1-D dam break on flat bathymetry or reads NetCDF
bathymetry through ASAGI (src/SWE/SWE_initialize.f90:120-185,349-370); the
workloads here are seeded synthetic generators of the same kind. Reference
depth d has 2^(d+1) cells (src/SFC_node_traversal.f90:46), so "2^k cells" is
reference depth k - 1. States are sampled at cell centroids; h is the surface
elevation (depth = h - b).
"""
from dataclasses import dataclass

import numpy as np

from .swe import Config, Grid, initial_dt, uniform_mesh


@dataclass
class Scenario:
    name: str
    grid: Grid
    cfg: Config
    steps: int


def _world(mesh, cfg):
    c = mesh.centroids
    return cfg.scaling * c[:, 0] + cfg.offset[0], cfg.scaling * c[:, 1] + cfg.offset[1]


def element_bathymetry(vertices, depth, max_depth, bathymetry, scaling, offset, chunk=1 << 20):
    """b of each cell as get_bathymetry_at_element computes it with _ADAPT_INTEGRATE
    (src/SWE/SWE_initialize.f90:105-147): the mean of ``bathymetry(x, y)`` over
    2^min(16, max_depth - depth) sub-triangles of the cell, each sampled at its
    centroid (x1 + x2 + x3) / 3 in world coordinates scaling * x + offset. The
    sub-triangles come from bisecting the hypotenuse: (x1, x2, x3), x2 the right
    angle, splits into (x1, m, x2) and (x2, m, x3), m = (x1 + x3) / 2; the mean is
    taken pairwise up the bisection tree, 0.5 * (first + second), as the
    reference's recursion does, so the rounding is the same. ``vertices`` is
    [n, 3, 2] in the unit square (the mesh builder's, right angle in the middle)."""
    vertices = np.asarray(vertices, np.float64)
    depth = np.asarray(depth)
    n = len(depth)
    out = np.empty(n, np.float64)
    dd = np.clip(max_depth - depth.astype(np.int64), 0, 16)
    for k in np.unique(dd):
        idx = np.nonzero(dd == k)[0]
        step = max(1, chunk >> int(k))
        for s in range(0, len(idx), step):
            sel = idx[s:s + step]
            v3 = vertices[sel]
            x1, x2, x3 = v3[:, None, 0], v3[:, None, 1], v3[:, None, 2]  # [m, 1, 2] each
            for _ in range(int(k)):
                mid = 0.5 * (x1 + x3)
                shape = (len(sel), 2 * x1.shape[1], 2)
                y1, y2, y3 = np.empty(shape), np.empty(shape), np.empty(shape)
                y1[:, 0::2], y2[:, 0::2], y3[:, 0::2] = x1, mid, x2  # first child (x1, m, x2)
                y1[:, 1::2], y2[:, 1::2], y3[:, 1::2] = x2, mid, x3  # second child (x2, m, x3)
                x1, x2, x3 = y1, y2, y3
            c = ((x1 + x2) + x3) / 3.0
            v = bathymetry(scaling * c[:, :, 0] + offset[0], scaling * c[:, :, 1] + offset[1])
            v = np.broadcast_to(np.asarray(v, np.float64), c.shape[:2])
            for _ in range(int(k)):
                v = 0.5 * (v[:, 0::2] + v[:, 1::2])
            out[sel] = v[:, 0]
    return out


def _vertices(mesh):
    """[n, 3, 2] vertices of a mesh's cells in the unit square (right angle in the middle)."""
    if mesh.vertices is not None:
        return mesh.vertices
    from .swe import mesh_from_depths
    return mesh_from_depths(mesh.depth, centroids=False, vertices=True).vertices


def _grid(mesh, cfg, h, b):
    n = mesh.n_cells
    hu = np.zeros(n)
    hv = np.zeros(n)
    g = Grid(mesh, np.ascontiguousarray(h, np.float64), hu, hv, np.ascontiguousarray(b, np.float64))
    g.r_dt = initial_dt(mesh, g.h, hu, hv, g.b, cfg.courant_number)
    return g


def radial_dam_break(log2_cells=16, boundary="slip", solver="fwave", mesh=None):
    """Radial dam break on [-0.5, 0.5]^2: flat b = -10 m, water depth 15 m inside
    r < 0.1 and 10 m elsewhere, at rest; CFL 0.5, 100 steps, no adaptivity."""
    d = log2_cells - 1
    cfg = Config(flux_solver=solver, boundary=boundary, courant_number=0.5, dry_tolerance=0.01, scaling=1.0,
                 offset=(-0.5, -0.5), i_min_depth=d, i_max_depth=d)
    mesh = mesh or uniform_mesh(d)
    x, y = _world(mesh, cfg)
    b = np.full(mesh.n_cells, -10.0)
    h = b + np.where(np.hypot(x, y) < 0.1, 15.0, 10.0)
    return Scenario("radial_dam_break", _grid(mesh, cfg, h, b), cfg, 100)


def apriori_mesh(cfg, surface, max_cells=1 << 26):
    """The a-priori refinement loop of the SWE initialisation (src/SWE/SWE.f90:232-269
    with the criteria of src/SWE/SWE_initialize.f90:292-322): starting from the two
    root cells, refine every cell shallower than the minimum depth, and every
    cell shallower than the maximum depth whose initial surface differs between
    its three vertices (the probes at barycentric (1,0), (0,0), (0,1)); remesh
    with conformity; repeat until no cell asks for refinement. `surface(x, y)`
    gives the initial surface at world points."""
    from .swe import adapt, mesh_from_depths
    mesh = mesh_from_depths(np.zeros(2, np.int8), vertices=True)
    while True:
        v = cfg.scaling * mesh.vertices + np.asarray(cfg.offset, np.float64)
        s = surface(v[:, :, 0], v[:, :, 1])
        d = mesh.depth
        want = (d < cfg.i_min_depth) | ((d < cfg.i_max_depth) & (s.max(axis=1) > s.min(axis=1)))
        if not want.any():
            return mesh
        mesh, _ = adapt(mesh, want.astype(np.int8))
        if mesh.n_cells > max_cells:
            raise ValueError("a-priori refinement exceeds %d cells" % max_cells)


def adaptive_dam_break(min_depth=6, max_depth=12, solver="fwave", boundary="outflow"):
    """The reference's default SWE initial state (src/SWE/SWE_initialize.f90:349-370):
    surface 1 m for x < 0 and 0 m elsewhere, at rest, over a flat bottom at -10 m,
    on the mesh of the a-priori refinement (max depth along the step, min depth
    elsewhere); dt from the initial CFL estimate."""
    cfg = Config(flux_solver=solver, boundary=boundary, courant_number=0.45, dry_tolerance=0.01, scaling=1.0,
                 offset=(-0.5, -0.5), i_min_depth=min_depth, i_max_depth=max_depth)
    surface = lambda x, y: np.where(x < 0.0, 1.0, 0.0)
    mesh = apriori_mesh(cfg, surface)
    x, y = _world(mesh, cfg)
    b = np.full(mesh.n_cells, -10.0)
    return Scenario("adaptive_dam_break", _grid(mesh, cfg, surface(x, y), b), cfg, 50)


def ci_dam_break(solver="llfbath", min_depth=0, max_depth=8):
    """The reference's own smoke run (.travis.yml:28-37: `-dmax 8 -nmax 10` with
    llfbath or aug_riemann): the default SWE scenario without ASAGI, i.e. the
    domain [-5, 5]^2 (scaling 10, src/SWE/SWE.f90:169-170), bathymetry 0
    (src/SWE/SWE_initialize.f90:186), surface 1 m for x < 0 and 0 m elsewhere
    (:349-370: dry land on the right), at rest; depths 0..8, Courant 0.45, dry
    tolerance 0.01 (src/Config.f90:183), a-priori refinement along the step."""
    cfg = Config(flux_solver=solver, boundary="outflow", courant_number=0.45, dry_tolerance=0.01, scaling=10.0,
                 offset=(-5.0, -5.0), i_min_depth=min_depth, i_max_depth=max_depth)
    surface = lambda x, y: np.where(x < 0.0, 1.0, 0.0)
    mesh = apriori_mesh(cfg, surface)
    x, y = _world(mesh, cfg)
    return Scenario("ci_dam_break", _grid(mesh, cfg, surface(x, y), np.zeros(mesh.n_cells)), cfg, 10)


def bowl_bathymetry(x, y, h0=10.0, a=0.4):
    r2 = x * x + y * y
    return -h0 * (1.0 - r2 / (a * a))


def parabolic_bowl(log2_cells=14, seed=2, solver="aug_riemann", amplitude=0.5, sigma=0.05, mesh=None,
                   min_depth=None, max_depth=None):
    """Parabolic bowl b(r) = -10 (1 - r^2 / 0.4^2) on [-0.5, 0.5]^2 (dry land for
    r > 0.4) with a Gaussian surface bump at a seeded offset; dry tolerance 1e-3 m.
    On a frozen uniform mesh (the remeshing of the adaptive case stays on the host).
    b is integrated over each cell as the initialisation does (element_bathymetry,
    down to the maximum depth); the surface is sampled at the centroid."""
    d = log2_cells - 1
    cfg = Config(flux_solver=solver, boundary="outflow", courant_number=0.45, dry_tolerance=1e-3, scaling=1.0,
                 offset=(-0.5, -0.5), i_min_depth=d if min_depth is None else min_depth,
                 i_max_depth=d + 1 if max_depth is None else max_depth)
    mesh = mesh or uniform_mesh(d)
    x, y = _world(mesh, cfg)
    rng = np.random.default_rng(seed)
    x0, y0 = rng.uniform(-0.1, 0.1, 2)
    b = element_bathymetry(_vertices(mesh), mesh.depth, cfg.i_max_depth, bowl_bathymetry, cfg.scaling, cfg.offset)
    eta = amplitude * np.exp(-((x - x0) ** 2 + (y - y0) ** 2) / (2 * sigma * sigma))
    # surface = eta over water; on land the state is dry: h = b (depth 0)
    h = np.where(b < eta, eta, b)
    return Scenario("parabolic_bowl", _grid(mesh, cfg, h, b), cfg, 500)


def adaptive_bowl(min_depth=12, max_depth=22, seed=2, solver="aug_riemann", amplitude=0.5, sigma=0.05):
    """The parabolic bowl on the mesh of the a-priori refinement between the given
    depths (the adaptive wet/dry configuration: the Gaussian surface differs
    between the vertices of every cell, so the initial mesh is uniform at the
    maximum depth; the flags of the step then coarsen the flat water). b is
    integrated over each cell (element_bathymetry), as refined cells get it
    during the run (run_adaptive with ``scn.bathymetry``)."""
    cfg = Config(flux_solver=solver, boundary="outflow", courant_number=0.45, dry_tolerance=1e-3, scaling=1.0,
                 offset=(-0.5, -0.5), i_min_depth=min_depth, i_max_depth=max_depth)
    rng = np.random.default_rng(seed)
    x0, y0 = rng.uniform(-0.1, 0.1, 2)
    eta_f = lambda x, y: amplitude * np.exp(-((x - x0) ** 2 + (y - y0) ** 2) / (2 * sigma * sigma))
    mesh = apriori_mesh(cfg, eta_f)
    x, y = _world(mesh, cfg)
    b = element_bathymetry(mesh.vertices, mesh.depth, max_depth, bowl_bathymetry, cfg.scaling, cfg.offset)
    eta = eta_f(x, y)
    h = np.where(b < eta, eta, b)
    scn = Scenario("adaptive_bowl", _grid(mesh, cfg, h, b), cfg, 500)
    scn.bathymetry = bowl_bathymetry
    return scn


def value_noise(x, y, seed, octaves=5, base=8.0, persistence=0.5):
    """Seeded lattice value noise in [-1, 1], smooth-step interpolated, summed over
    octaves (frequency doubling, amplitude times ``persistence``). x, y in [-0.5, 0.5]."""
    rng = np.random.default_rng(seed)
    out = np.zeros_like(x)
    amp, freq, norm = 1.0, base, 0.0
    for _ in range(octaves):
        k = int(freq) + 3
        table = rng.uniform(-1.0, 1.0, (k, k))
        fx = (x + 0.5) * freq
        fy = (y + 0.5) * freq
        ix = np.clip(np.floor(fx).astype(np.int64), 0, k - 2)
        iy = np.clip(np.floor(fy).astype(np.int64), 0, k - 2)
        tx = fx - ix
        ty = fy - iy
        sx = tx * tx * (3.0 - 2.0 * tx)
        sy = ty * ty * (3.0 - 2.0 * ty)
        flat = table.ravel()
        base_i = ix * k + iy
        v00, v10 = flat[base_i], flat[base_i + k]
        v01, v11 = flat[base_i + 1], flat[base_i + k + 1]
        a = v00 + sx * (v10 - v00)
        b = v01 + sx * (v11 - v01)
        out += amp * (a + sy * (b - a))
        norm += amp
        amp *= persistence
        freq *= 2.0
    out /= norm
    return out


def _value_noise_torch(u, v, seed, octaves=5, base=8.0, persistence=0.5):
    """value_noise() evaluated with torch (multi-threaded on the CPU, or on a GPU)."""
    import torch
    rng = np.random.default_rng(seed)
    out = torch.zeros_like(u)
    amp, freq, norm = 1.0, base, 0.0
    for _ in range(octaves):
        k = int(freq) + 3
        flat = torch.as_tensor(rng.uniform(-1.0, 1.0, (k, k)).ravel(), dtype=u.dtype, device=u.device)
        fx = (u + 0.5) * freq
        fy = (v + 0.5) * freq
        ix = torch.clamp(torch.floor(fx), 0, k - 2)
        iy = torch.clamp(torch.floor(fy), 0, k - 2)
        tx, ty = fx - ix, fy - iy
        sx = tx * tx * (3.0 - 2.0 * tx)
        sy = ty * ty * (3.0 - 2.0 * ty)
        bi = (ix * k + iy).long()
        v00, v10, v01, v11 = flat[bi], flat[bi + k], flat[bi + 1], flat[bi + k + 1]
        a = v00 + sx * (v10 - v00)
        b = v01 + sx * (v11 - v01)
        out += amp * (a + sy * (b - a))
        norm += amp
        amp *= persistence
        freq *= 2.0
    return out / norm


def ocean_basin(log2_cells=26, seed=3, solver="fwave", steps=200, mesh=None, scaling=1.0e6, device="cpu"):
    """Synthetic ocean basin: tanh shelf from a -4000 m abyssal plain to a -50 m
    shelf plus 200 m of 5-octave seeded value noise, a Gaussian uplift of 2 m
    with sigma 2 % of the domain width at a seeded centre; f-wave, outflow.
    The fields are evaluated with torch on ``device`` (the mesh can have 2^26 cells)."""
    import torch
    d = log2_cells - 1
    cfg = Config(flux_solver=solver, boundary="outflow", courant_number=0.45, dry_tolerance=0.01, scaling=scaling,
                 offset=(-0.5 * scaling, -0.5 * scaling), i_min_depth=d, i_max_depth=d)
    mesh = mesh or uniform_mesh(d)
    cen = torch.from_numpy(mesh.centroids).to(device)
    u = cen[:, 0] - 0.5
    v = cen[:, 1] - 0.5
    rng = np.random.default_rng(seed)
    x0, y0 = (float(t) for t in rng.uniform(-0.25, 0.1, 2))
    b = -4000.0 + 3950.0 * 0.5 * (1.0 + torch.tanh((u - 0.25) / 0.05)) + 200.0 * _value_noise_torch(u, v, seed)
    b = torch.clamp(b, max=-20.0)  # keep the shelf under water
    eta = 2.0 * torch.exp(-((u - x0) ** 2 + (v - y0) ** 2) / (2 * 0.02 * 0.02))
    h = eta.cpu().numpy()
    b = b.cpu().numpy()
    return Scenario("ocean_basin", _grid(mesh, cfg, h, b), cfg, steps)


def current_basin(log2_cells=12, u0=2.0, v0=1.0, seed=8, mesh=None):
    """A deep basin (100 km square, depths 80 to 120 m of smooth seeded relief)
    under a uniform current (u0, v0) m/s with a 0.5 m Gaussian surface bump: all
    wet, and the normal velocity is away from 0 on every edge orientation of the
    Sierpinski mesh (axis-aligned and diagonal normals), so no wave speed sits
    at 0. f-wave, outflow. Returns the scenario with the current's momenta set."""
    d = log2_cells - 1
    cfg = Config(flux_solver="fwave", boundary="outflow", courant_number=0.45, dry_tolerance=0.01, scaling=1.0e5,
                 offset=(-0.5e5, -0.5e5), i_min_depth=d, i_max_depth=d)
    mesh = mesh or uniform_mesh(d)
    u, v = mesh.centroids[:, 0] - 0.5, mesh.centroids[:, 1] - 0.5
    b = -100.0 + 20.0 * value_noise(u, v, seed, octaves=2, base=3.0)
    h = 0.5 * np.exp(-(u * u + v * v) / (2 * 0.1 * 0.1))
    g = _grid(mesh, cfg, h, b)
    depth = g.h - g.b
    g.hu[:] = depth * u0
    g.hv[:] = depth * v0
    g.r_dt = initial_dt(mesh, g.h, g.hu, g.hv, g.b, cfg.courant_number)
    return Scenario("current_basin", g, cfg, 100)


def lake_at_rest(log2_cells=10, solver="fwave", seed=7, mesh=None):
    """Flat surface at 0 over rough bathymetry, at rest: the well-balanced solvers keep it exactly."""
    d = log2_cells - 1
    cfg = Config(flux_solver=solver, boundary="outflow", courant_number=0.45, dry_tolerance=0.01, scaling=1.0,
                 offset=(-0.5, -0.5), i_min_depth=0, i_max_depth=d + 1)
    mesh = mesh or uniform_mesh(d)
    x, y = _world(mesh, cfg)
    b = -5.0 + 2.0 * value_noise(x, y, seed, octaves=3)
    h = np.zeros(mesh.n_cells)
    return Scenario("lake_at_rest", _grid(mesh, cfg, h, b), cfg, 10)


@dataclass
class Ensemble:
    name: str
    meshes: list
    grids: list
    cfgs: list
    steps: int


def bowl_ensemble(n_instances=512, seed=4, log2_range=(12, 20), solver="fwave", steps=1000, device="cpu"):
    """Ensemble of independent parabolic-bowl instances: uniform meshes of 2^k
    cells with k uniform in ``log2_range`` (4k..1M cells), the bowl bathymetry,
    a Gaussian surface bump per instance with amplitude U[0.5, 3] m, sigma
    U[0.03, 0.08] and a seeded centre; f-wave, CFL 0.5, each with its own dt."""
    import torch
    rng = np.random.default_rng(seed)
    ks = rng.integers(log2_range[0], log2_range[1] + 1, n_instances)
    amps = rng.uniform(0.5, 3.0, n_instances)
    sigmas = rng.uniform(0.03, 0.08, n_instances)
    centres = rng.uniform(-0.15, 0.15, (n_instances, 2))
    cache = {}
    meshes, grids, cfgs = [], [], []
    for i in range(n_instances):
        k = int(ks[i])
        if k not in cache:
            cache[k] = uniform_mesh(k - 1)
        mesh = cache[k]
        cfg = Config(flux_solver=solver, boundary="outflow", courant_number=0.5, dry_tolerance=1e-3, scaling=1.0,
                     offset=(-0.5, -0.5), i_min_depth=k - 1, i_max_depth=k - 1)
        cen = torch.from_numpy(mesh.centroids).to(device)
        x = cen[:, 0] - 0.5
        y = cen[:, 1] - 0.5
        b = -10.0 * (1.0 - (x * x + y * y) / 0.16)
        eta = amps[i] * torch.exp(-((x - centres[i, 0]) ** 2 + (y - centres[i, 1]) ** 2) / (2 * sigmas[i] ** 2))
        h = torch.where(b < eta, eta, b)
        g = _grid(mesh, cfg, h.cpu().numpy(), b.cpu().numpy())
        meshes.append(mesh)
        grids.append(g)
        cfgs.append(cfg)
    return Ensemble("bowl_ensemble", meshes, grids, cfgs, steps)


def adjoint_case(log2_cells=18, steps=2000, n_gauges=32, seed=5, device=0):
    """Gauge-misfit problem: the deep basin bathymetry (always wet), a Gaussian
    source of 2 m, 32 gauges at seeded deep-water cells, observations from a
    forward run of a seeded perturbed source (amplitude and centre), and the
    CFL dt sequence of the unperturbed run, frozen. Returns a dict with mesh,
    params, h0, b, gauges, obs, dts and the perturbed source."""
    import torch

    from .adjoint import GaugeProblem, record_dts
    base = ocean_basin(log2_cells=log2_cells, seed=seed, steps=steps)
    mesh, cfg = base.grid.mesh, base.cfg
    b = base.grid.b
    params = cfg.params()
    rng = np.random.default_rng(seed)
    deep = np.nonzero(b < -1000.0)[0]
    gauges = np.sort(rng.choice(deep, n_gauges, replace=False))
    u = mesh.centroids[:, 0] - 0.5
    v = mesh.centroids[:, 1] - 0.5
    x0, y0 = rng.uniform(-0.25, 0.0, 2)
    h0 = 2.0 * np.exp(-((u - x0) ** 2 + (v - y0) ** 2) / (2 * 0.02 ** 2))
    amp, dx, dy = rng.uniform(1.1, 1.3), rng.uniform(-0.01, 0.01), rng.uniform(-0.01, 0.01)
    h_obs = amp * 2.0 * np.exp(-((u - x0 - dx) ** 2 + (v - y0 - dy) ** 2) / (2 * 0.02 ** 2))
    dts = record_dts(mesh, params, h0, b, steps, device=device)
    P = GaugeProblem(mesh, params, gauges, np.zeros((steps, n_gauges)), dts, snapshots=1, device=device)
    try:
        P.objective(h_obs, b)
        obs = P.gauge_values.cpu().numpy().copy()
    finally:
        P.close()
    return dict(mesh=mesh, cfg=cfg, params=params, h0=h0, b=b, gauges=gauges, obs=obs, dts=dts, h_obs=h_obs)
