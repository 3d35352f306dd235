"""Generate the golden fixtures of the SWE step (run from the repository root:
``python -m tests.golden.make_golden``).

The reference (sam(oa)², Fortran) cannot be built or run here and ships no
golden vectors for this path, so these fixtures are produced by the oracle,
the strict-IEEE C restatement of the reference step (oracle/swe_oracle.c),
and frozen. They pin the oracle and the GPU path to fixed answers:

* ``riemann_kat.npz`` — solver-level known answers: 512 edge states (wet/wet,
  dry/dry, wet/dry, walls, water at rest, equal depths, identical states, slow
  flow; random normals) and the edge fluxes (both sides: h, hu, hv, max wave
  speed) of every solver, from ``oracle.edge_flux``. The LF and LLF fluxes
  without bathymetry take the surface as the depth (the reference assumes
  b = 0 for them), so they get the same states moved to a flat bottom, all
  wet (``ql_flat``, ``qr_flat``: b = 0, surface = |depth| + 1).
* ``ci_smoke_<solver>.npz`` — the reference's own CI smoke run
  (.travis.yml:28-37: the default SWE scenario, ``-dmax 8 -nmax 10``, for
  llfbath and aug_riemann): the a-priori refined mesh, then 10 steps, each
  after a remesh from the previous step's flags (src/SWE/SWE.f90:378-392).
  The oracle walks each step; the remesh is the library's host adaption
  (swe_mesh_adapt). Per step: cells, time, dt, dt_new, refinements and a
  SHA-256 of (h, hu, hv, flags) with -0 mapped to +0; the final mesh and state.
"""
import hashlib
import os

import numpy as np

from oracle import oracle as O
from samoa_gb300 import scenarios, swe

HERE = os.path.dirname(os.path.abspath(__file__))
KAT_SOLVERS = ("fwave", "aug_riemann", "lf", "lfbath", "llf", "llfbath")
SMOKE_SOLVERS = ("llfbath", "aug_riemann")


def digest(h, hu, hv, flags):
    m = hashlib.sha256()
    for a in (h, hu, hv):
        m.update((np.asarray(a, np.float64) + 0.0).tobytes())
    m.update(np.asarray(flags, np.int8).tobytes())
    return m.hexdigest()


def kat_states(n=512, seed=11):
    """Edge states: random wet/dry pairs plus degenerate families."""
    rng = np.random.default_rng(seed)
    normals = rng.normal(size=(n, 2))
    normals /= np.linalg.norm(normals, axis=1, keepdims=True)
    normals[:32] = [[1.0, 0.0], [0.0, 1.0], [-1.0, 0.0], [0.0, -1.0]] * 8  # axis-aligned
    bl = rng.uniform(-20, 5, n)
    br = bl + rng.choice([0.0, 1.0], n) * rng.uniform(-10, 10, n)
    dl = rng.choice([0.0, 1e-4, 1.0], n, p=[0.2, 0.1, 0.7]) * rng.uniform(0, 20, n)
    dr = rng.choice([0.0, 1e-4, 1.0], n, p=[0.2, 0.1, 0.7]) * rng.uniform(0, 20, n)
    ql = np.stack([bl + dl, rng.normal(0, 30, n), rng.normal(0, 30, n), bl], 1)
    qr = np.stack([br + dr, rng.normal(0, 30, n), rng.normal(0, 30, n), br], 1)
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
    return normals, ql, qr


FLAT_SOLVERS = ("lf", "llf")


def flat(q):
    """The states over a flat bottom, all wet: surface = |depth| + 1, b = 0."""
    f = q.copy()
    f[:, 0] = np.abs(q[:, 0] - q[:, 3]) + 1.0
    f[:, 3] = 0.0
    return f


def kat_fluxes(solver, normals, ql, qr, drytol):
    n = len(normals)
    fl, fr = np.zeros((n, 4)), np.zeros((n, 4))
    for i in range(n):
        fl[i], fr[i] = O.edge_flux(swe.SOLVERS[solver], normals[i], ql[i], qr[i], drytol)
    return fl, fr


def smoke_run(solver, steps=10):
    """The CI smoke run on the oracle: returns the per-step records and the final mesh and state."""
    from tests.helpers import oracle_params
    scn = scenarios.ci_dam_break(solver)
    g = scn.grid
    P = oracle_params(scn.cfg)
    mesh, h, hu, hv, b, t, dt = g.mesh, g.h, g.hu, g.hv, g.b, g.r_time, g.r_dt
    rec = {"cells": [], "time": [], "dt": [], "dt_new": [], "refinements": [], "digest": []}
    flags = None
    for k in range(steps):
        if k > 0:
            mesh, (h, hu, hv, b) = swe.adapt(mesh, flags, h, hu, hv, b)
        o = O.mesh_from_depths(mesh.depth)
        W = O.WalkState(o["cells5"], h, hu, hv, b, t, dt)
        W.steps(P, 1)
        h, hu, hv, flags = W.h.copy(), W.hu.copy(), W.hv.copy(), W.flags.copy()
        t, dt = W.time, W.dt
        rec["cells"].append(mesh.n_cells)
        rec["time"].append(t)
        rec["dt"].append(dt)
        rec["dt_new"].append(W.dt_new)
        rec["refinements"].append(W.n_refine)
        rec["digest"].append(digest(h, hu, hv, flags))
    return scn, rec, (mesh.depth.copy(), h, hu, hv, b, flags)


def main():
    drytol = 1e-3
    normals, ql, qr = kat_states()
    out = {"normals": normals, "ql": ql, "qr": qr, "ql_flat": flat(ql), "qr_flat": flat(qr),
           "drytol": np.float64(drytol)}
    for s in KAT_SOLVERS:
        a, b = (out["ql_flat"], out["qr_flat"]) if s in FLAT_SOLVERS else (ql, qr)
        out["fl_" + s], out["fr_" + s] = kat_fluxes(s, normals, a, b, drytol)
    np.savez_compressed(os.path.join(HERE, "riemann_kat.npz"), **out)
    for s in SMOKE_SOLVERS:
        scn, rec, (depth, h, hu, hv, b, flags) = smoke_run(s)
        g = scn.grid
        np.savez_compressed(os.path.join(HERE, "ci_smoke_%s.npz" % s),
                            depth0=g.mesh.depth, h0=g.h, b0=g.b, dt0=np.float64(g.r_dt),
                            cells=np.array(rec["cells"]), time=np.array(rec["time"]), dt=np.array(rec["dt"]),
                            dt_new=np.array(rec["dt_new"]), refinements=np.array(rec["refinements"]),
                            digest=np.array(rec["digest"]), depth=depth, h=h, hu=hu, hv=hv, b=b, flags=flags)
        print(s, rec["cells"], rec["refinements"])


if __name__ == "__main__":
    main()
