"""swe_step_host: the step reading and writing the caller's arrays in pinned
host memory (or device memory) equals the resident-state step bit for bit,
including the refinement flags, the dt and the traversal direction."""
import numpy as np
import pytest

from samoa_gb300 import scenarios, swe

pytestmark = pytest.mark.gpu


def _dt0(scn):
    g = scn.grid
    return swe.initial_dt(g.mesh, g.h, g.hu, g.hv, g.b, scn.cfg.courant_number)


def _resident(scn, steps):
    ctx = swe.SweContext(0)
    try:
        ctx.set_params(scn.cfg.params())
        ctx.upload_mesh(scn.grid.mesh)
        g = scn.grid
        ctx.upload_state(g.h, g.hu, g.hv, g.b)
        ctx.set_time(0.0, _dt0(scn))
        out = []
        for _ in range(steps):
            ctx.traverse(1)
            h, hu, hv, _ = ctx.download_state()
            flags, n = ctx.refinements()
            out.append((h, hu, hv, flags.copy(), n, ctx.get_time()))
        return out
    finally:
        ctx.close()


@pytest.mark.parametrize("where,cross", [("pinned", "auto"), ("device", "auto"), ("device_offset", "auto"),
                                         ("pinned", "pass"), ("device", "inkernel"), ("pinned_b_resident", "auto")])
def test_host_step_matches_resident_step(swe_lib, where, cross):
    """The step on the caller's arrays (pinned host memory, device memory, 8-byte
    aligned device memory; b passed each step, or b = NULL: the uploaded
    bathymetry) against the resident step, bit for bit."""
    import torch
    scn = scenarios.radial_dam_break(log2_cells=12, boundary="slip")
    g = scn.grid
    steps = 3
    ref = _resident(scn, steps)
    n = g.mesh.n_cells
    b_resident = where == "pinned_b_resident"
    if where in ("pinned", "pinned_b_resident"):
        mk = lambda a: torch.tensor(a).pin_memory()
        buf = lambda dt: torch.zeros(n, dtype=dt).pin_memory()
    elif where == "device":
        mk = lambda a: torch.tensor(a, device="cuda")
        buf = lambda dt: torch.zeros(n, dtype=dt, device="cuda")
    else:  # 8-byte aligned bases: the plain-load staging path
        mk = lambda a: torch.tensor(np.concatenate([[0.0], a]), device="cuda")[1:]
        buf = lambda dt: torch.zeros(n + 1, dtype=dt, device="cuda")[1:]
    cur = [mk(g.h), mk(g.hu), mk(g.hv)]
    nxt = [buf(torch.float64) for _ in range(3)]
    b = mk(g.b)
    flags = buf(torch.int8)
    ctx = swe.SweContext(0)
    try:
        ctx.set_params(scn.cfg.params())
        ctx.upload_mesh(g.mesh)
        ctx.set_cross_pass(cross)
        if b_resident:
            ctx.upload_state(g.h, g.hu, g.hv, g.b)
        ctx.set_time(0.0, _dt0(scn))
        for k in range(steps):
            ctx.step_host(*cur, None if b_resident else b, *nxt, flags)
            ctx.synchronize()
            h, hu, hv, f, nref, tm = ref[k]
            assert np.array_equal(nxt[0].cpu().numpy(), h)
            assert np.array_equal(nxt[1].cpu().numpy(), hu)
            assert np.array_equal(nxt[2].cpu().numpy(), hv)
            assert np.array_equal(flags.cpu().numpy(), f)
            assert ctx.get_time() == tm
            cur, nxt = nxt, cur
    finally:
        ctx.close()


def test_host_step_rejects_overlap_and_pageable_policy(swe_lib):
    import torch
    from samoa_gb300 import _lib
    scn = scenarios.radial_dam_break(log2_cells=10, boundary="outflow")
    g = scn.grid
    n = g.mesh.n_cells
    ctx = swe.SweContext(0)
    try:
        ctx.set_params(scn.cfg.params())
        ctx.upload_mesh(g.mesh)
        ctx.set_time(0.0, _dt0(scn))
        a = torch.zeros(4 * n, dtype=torch.float64).pin_memory()
        b = torch.tensor(g.b).pin_memory()
        with pytest.raises(_lib.SweError):  # h_out overlaps h and hu
            ctx.step_host(a[:n], a[n:2 * n], a[2 * n:3 * n], b, a[n // 2:n // 2 + n], a[3 * n:], a[3 * n:])
        with pytest.raises(_lib.SweError):  # no bathymetry anywhere
            ctx.step_host(a[:n], a[n:2 * n], a[2 * n:3 * n], None, *[torch.zeros(n, dtype=torch.float64).pin_memory()
                                                                    for _ in range(3)])
    finally:
        ctx.close()


def test_host_step_on_pageable_memory(swe_lib):
    """Plain (pageable) numpy arrays: on a device with coherent pageable memory
    access (Grace) the step reads and writes them in place, bit-exact with the
    resident step; elsewhere the call is refused with a message, not a fault."""
    import ctypes as C
    from samoa_gb300 import _lib
    scn = scenarios.radial_dam_break(log2_cells=10, boundary="slip")
    g = scn.grid
    ref = _resident(scn, 1)
    h, hu, hv, b = (np.array(a, np.float64) for a in (g.h, g.hu, g.hv, g.b))
    out = [np.zeros_like(h) for _ in range(3)]
    flags = np.zeros(g.mesh.n_cells, np.int8)
    ctx = swe.SweContext(0)
    try:
        ctx.set_params(scn.cfg.params())
        ctx.upload_mesh(g.mesh)
        ctx.set_time(0.0, _dt0(scn))
        p = lambda a: a.ctypes.data_as(C.c_void_p)
        rc = ctx.L.swe_step_host(ctx.ptr, p(h), p(hu), p(hv), p(b), p(out[0]), p(out[1]), p(out[2]), p(flags))
        if rc != 0:
            assert "pageable" in _lib.last_error()
            return
        ctx.synchronize()
        rh, rhu, rhv, rf, _, _ = ref[0]
        assert np.array_equal(out[0], rh) and np.array_equal(out[1], rhu) and np.array_equal(out[2], rhv)
        assert np.array_equal(flags, rf)
    finally:
        ctx.close()
