"""Failure detection on the GPU, in the forms that fault nothing.

The step kernel waits for its bulk copies on an mbarrier with a bounded wait
(global-timer limit): when the wait gives up, the CTA leaves its segment, the
kernel records the error and returns, and the host reports SWE_E_DEVICE. The
test-only injection SWE_INJECT_STAGING_TX arms the staging barrier for 16 bytes
that no copy delivers, so every issued copy lands but the phase never
completes and the wait runs out (20 ms limit under injection). The tests check
the reported status and that the same context then steps bit for bit like the
oracle again, once a state is uploaded.
"""
import numpy as np
import pytest

from samoa_gb300 import _lib, scenarios, swe

from .helpers import assert_state_equal, omp_state, oracle_params

pytestmark = pytest.mark.gpu

SWE_E_DEVICE = -6
SWE_INJECT_NONE, SWE_INJECT_STAGING_TX = 0, 1


def _ctx_with(scn):
    g = scn.grid
    ctx = swe.SweContext(0)
    ctx.set_params(scn.cfg.params())
    ctx.upload_mesh(g.mesh)
    ctx.upload_state(g.h, g.hu, g.hv, g.b)
    ctx.set_time(0.0, g.r_dt)
    return ctx


@pytest.mark.parametrize("staging", [1, 2])
def test_staging_wait_runs_out_and_context_recovers(swe_lib, oracle_lib, staging):
    scn = scenarios.radial_dam_break(log2_cells=14, boundary="outflow")
    g = scn.grid
    ctx = _ctx_with(scn)
    try:
        ctx.set_staging(staging)
        L = _lib.load()
        _lib.check(L.swe_set_fault_injection(ctx.ptr, SWE_INJECT_STAGING_TX))
        ctx.traverse(1)
        with pytest.raises(_lib.SweError) as err:
            ctx.synchronize()
        assert err.value.code == SWE_E_DEVICE and "wait ran out" in str(err.value)
        # reported once: the device flag is clear again
        ctx.synchronize()

        _lib.check(L.swe_set_fault_injection(ctx.ptr, SWE_INJECT_NONE))
        ctx.upload_mesh(g.mesh)
        ctx.upload_state(g.h, g.hu, g.hv, g.b)
        ctx.set_time(0.0, g.r_dt)
        O = omp_state(g.mesh, g)
        P = oracle_params(scn.cfg)
        for k in range(4):
            ctx.traverse(1)
            ctx.synchronize()
            O.steps(P, 1)
            h, hu, hv, _ = ctx.download_state()
            assert_state_equal("after recovery, step %d" % k, h, hu, hv, O.h, O.hu, O.hv)
            flags, nref = ctx.refinements()
            assert np.array_equal(flags, O.flags) and nref == O.n_refine
    finally:
        ctx.close()


def test_fault_injection_rejects_unknown_kind(swe_lib):
    scn = scenarios.radial_dam_break(log2_cells=8, boundary="outflow")
    ctx = _ctx_with(scn)
    try:
        rc = _lib.load().swe_set_fault_injection(ctx.ptr, 7)
        assert rc == -1
    finally:
        ctx.close()
