"""The committed golden fixtures (tests/golden/, made by make_golden.py from the
oracle): the oracle and the scenario generator reproduce them on the CPU, and
the GPU path reproduces them through the C ABI (solver-level known answers,
and the reference's CI smoke run with a remesh before every step)."""
import ctypes as C
import os

import numpy as np
import pytest

from samoa_gb300 import _lib, scenarios, swe

from .golden import make_golden as MG
from .helpers import same_bits

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _load(name):
    with np.load(os.path.join(GOLDEN, name)) as z:
        return {k: z[k] for k in z.files}


def test_oracle_reproduces_riemann_kat(oracle_lib):
    K = _load("riemann_kat.npz")
    normals, ql, qr = MG.kat_states()
    assert np.array_equal(normals, K["normals"]) and np.array_equal(ql, K["ql"]) and np.array_equal(qr, K["qr"])
    assert np.array_equal(MG.flat(ql), K["ql_flat"]) and np.array_equal(MG.flat(qr), K["qr_flat"])
    for s in MG.KAT_SOLVERS:
        a, b = (K["ql_flat"], K["qr_flat"]) if s in MG.FLAT_SOLVERS else (K["ql"], K["qr"])
        fl, fr = MG.kat_fluxes(s, K["normals"], a, b, float(K["drytol"]))
        assert np.isfinite(K["fl_" + s]).all() and np.isfinite(K["fr_" + s]).all(), s
        assert same_bits(fl, K["fl_" + s]) and same_bits(fr, K["fr_" + s]), s


@pytest.mark.parametrize("solver", MG.SMOKE_SOLVERS)
def test_ci_scenario_matches_fixture_inputs(swe_lib, solver):
    G = _load("ci_smoke_%s.npz" % solver)
    g = scenarios.ci_dam_break(solver).grid
    assert np.array_equal(g.mesh.depth, G["depth0"]) and same_bits(g.h, G["h0"]) and same_bits(g.b, G["b0"])
    assert g.r_dt == float(G["dt0"])


@pytest.mark.parametrize("solver", MG.SMOKE_SOLVERS)
def test_oracle_reproduces_ci_smoke(swe_lib, oracle_lib, solver):
    G = _load("ci_smoke_%s.npz" % solver)
    _, rec, (depth, h, hu, hv, b, flags) = MG.smoke_run(solver)
    assert list(G["cells"]) == rec["cells"] and list(G["refinements"]) == rec["refinements"]
    assert list(G["time"]) == rec["time"] and list(G["dt"]) == rec["dt"] and list(G["dt_new"]) == rec["dt_new"]
    assert list(G["digest"]) == rec["digest"]
    assert np.array_equal(depth, G["depth"]) and np.array_equal(flags, G["flags"])
    for a, k in ((h, "h"), (hu, "hu"), (hv, "hv"), (b, "b")):
        assert same_bits(a, G[k]), k


@pytest.mark.gpu
def test_gpu_riemann_batch_matches_kat(swe_lib):
    K = _load("riemann_kat.npz")
    L = _lib.load()
    p = lambda a: np.ascontiguousarray(a).ctypes.data_as(C.c_void_p)
    n = len(K["normals"])
    for s in MG.KAT_SOLVERS:
        a, b = (K["ql_flat"], K["qr_flat"]) if s in MG.FLAT_SOLVERS else (K["ql"], K["qr"])
        gl, gr = np.zeros((n, 4)), np.zeros((n, 4))
        _lib.check(L.swe_riemann_batch(swe.SOLVERS[s], n, p(K["normals"]), p(a), p(b), float(K["drytol"]),
                                       p(gl), p(gr)))
        assert same_bits(gl, K["fl_" + s]) and same_bits(gr, K["fr_" + s]), s


@pytest.mark.gpu
@pytest.mark.parametrize("solver", MG.SMOKE_SOLVERS)
def test_gpu_ci_smoke_matches_golden(swe_lib, solver):
    """The CI smoke run on the GPU: each step through the context (upload, one
    traverse, download), each remesh by the host adaption, every step's digest,
    scalars and the final state equal to the fixture."""
    G = _load("ci_smoke_%s.npz" % solver)
    scn = scenarios.ci_dam_break(solver)
    g = scn.grid
    mesh, h, hu, hv, b, t, dt = g.mesh, g.h, g.hu, g.hv, g.b, g.r_time, g.r_dt
    ctx = swe.SweContext(0)
    flags = None
    try:
        ctx.set_params(scn.cfg.params())
        for k in range(len(G["cells"])):
            if k > 0:
                mesh, (h, hu, hv, b) = swe.adapt(mesh, flags, h, hu, hv, b)
            ctx.upload_mesh(mesh)
            ctx.upload_state(h, hu, hv, b)
            ctx.set_time(t, dt)
            ctx.traverse(1)
            h, hu, hv, _ = ctx.download_state()
            flags, nref = ctx.refinements()
            t, dt, dt_new = ctx.get_time()
            tag = "%s step %d" % (solver, k)
            assert mesh.n_cells == G["cells"][k] and nref == G["refinements"][k], tag
            assert (t, dt, dt_new) == (G["time"][k], G["dt"][k], G["dt_new"][k]), tag
            assert MG.digest(h, hu, hv, flags) == G["digest"][k], tag
        assert np.array_equal(mesh.depth, G["depth"]) and np.array_equal(flags, G["flags"])
        for a, key in ((h, "h"), (hu, "hu"), (hv, "hv"), (b, "b")):
            assert same_bits(a, G[key]), key
    finally:
        ctx.close()
