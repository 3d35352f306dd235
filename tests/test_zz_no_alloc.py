"""swe_step_noalloc: the step for callers that cannot allocate device memory.

Such a caller owns all device buffers (for example a host code that takes all
its device memory from its own pool); the entry point keeps its scratch in a
fixed array inside the library. This test drives it through the C ABI on
buffers the test allocates with torch, for two calls in a row (parity 0, then
1), and checks each call's state, flags, dt_new and refinement count against
the context-based entry point (swe_traverse) on the same inputs: the
arithmetic is the same, so they must agree bit for bit. Collected last, so a
failure here comes after every other test has run.
"""
import ctypes as C

import numpy as np
import pytest

from samoa_gb300 import _lib, scenarios, swe

pytestmark = pytest.mark.gpu


def _ptr(t):
    return C.c_void_p(t.data_ptr())


def test_noalloc_step_matches_context_step(swe_lib):
    import torch
    scn = scenarios.parabolic_bowl(log2_cells=12, solver="fwave", amplitude=2.0, sigma=0.08, min_depth=6,
                                   max_depth=13)
    g = scn.grid
    m = g.mesh
    n = m.n_cells
    params = scn.cfg.params()

    # reference: the context entry point, two steps, state read back after each
    ctx = swe.SweContext(0)
    ctx.set_params(params)
    ctx.upload_mesh(m)
    ctx.upload_state(g.h, g.hu, g.hv, g.b)
    ctx.set_time(0.0, g.r_dt)
    ref = []
    for _ in range(2):
        _, dt, _ = ctx.get_time()
        ctx.traverse(1)
        ctx.synchronize()
        h, hu, hv, _ = ctx.download_state()
        flags, nref = ctx.refinements()
        _, _, dt_new = ctx.get_time()
        ref.append((dt, h, hu, hv, flags.copy(), nref, dt_new))
    ctx.close()

    dev = torch.device("cuda", 0)
    t = lambda a, dt: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=dev)
    depth = t(m.depth, torch.int8)
    plotter = t(m.plotter, torch.int8)
    ec = t(m.edge_cells.reshape(-1), torch.int64)
    el = t(m.edge_local.reshape(-1), torch.int8)
    bc = t(m.bnd_cell, torch.int64)
    bl = t(m.bnd_local, torch.int8)
    state = [t(g.h, torch.float64), t(g.hu, torch.float64), t(g.hv, torch.float64)]
    b = t(g.b, torch.float64)
    out = [torch.empty(n, dtype=torch.float64, device=dev) for _ in range(3)]
    flags = torch.empty(n, dtype=torch.int8, device=dev)
    dt_new = torch.empty(1, dtype=torch.float64, device=dev)
    nref = torch.empty(1, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    L = _lib.load()
    for k in range(2):
        dt = ref[k][0]
        rc = L.swe_step_noalloc(C.byref(params), n, _ptr(depth), _ptr(plotter), len(m.edge_cells), _ptr(ec),
                                _ptr(el), len(m.bnd_cell), _ptr(bc), _ptr(bl), _ptr(state[0]), _ptr(state[1]),
                                _ptr(state[2]), _ptr(b), _ptr(out[0]), _ptr(out[1]), _ptr(out[2]), _ptr(flags),
                                C.c_double(dt), k, _ptr(dt_new), _ptr(nref), C.c_void_p(stream))
        _lib.check(rc)
        torch.cuda.synchronize()
        _, h, hu, hv, f, nr, dn = ref[k]
        for got, want in zip(out, (h, hu, hv)):
            assert np.array_equal(got.cpu().numpy(), want), "call %d: state differs" % k
        assert np.array_equal(flags.cpu().numpy(), f), "call %d: flags differ" % k
        assert int(nref.item()) == nr and float(dt_new.item()) == dn, "call %d" % k
        state, out = out, state


def test_noalloc_rejects_oversized_mesh(swe_lib):
    params = swe.Config().params()
    rc = _lib.load().swe_step_noalloc(C.byref(params), 1 << 17, *([None] * 2), 0, None, None, 3 << 17, None, None,
                                      *([None] * 8), C.c_double(0.1), 0, None, None, None)
    assert rc == -1 and "65536" in _lib.last_error()
