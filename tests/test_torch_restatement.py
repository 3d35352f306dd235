"""The FP64 torch restatement (the reference gradient of the discrete adjoint)
against the oracle: its forward step equals the oracle's bit for bit for every
solver it restates, on wet/dry and wall cases, on both traversal parities."""
import numpy as np
import pytest

from oracle import swe_torch as ST
from samoa_gb300 import scenarios

from .helpers import omp_state, oracle_params, random_states_scenario


def _case(name, solver):
    if name == "random":
        scn = random_states_scenario(solver)
    elif name == "bowl":
        scn = scenarios.parabolic_bowl(log2_cells=10, solver=solver, amplitude=2.5, sigma=0.08)
    else:
        scn = scenarios.radial_dam_break(log2_cells=10, boundary="slip", solver=solver)
    if solver in ("lf", "llf"):  # the fluxes without bathymetry take the surface as the depth: b = 0, all wet
        g = scn.grid
        g.h[:] = (g.h - g.b) + 1.0
        g.b[:] = 0.0
        scn.cfg.courant_number = 0.05
    return scn


@pytest.mark.parametrize("solver", ["fwave", "aug_riemann", "lfbath", "llfbath", "lf", "llf"])
@pytest.mark.parametrize("name", ["bowl", "dam", "random"])
def test_torch_step_equals_oracle(oracle_lib, solver, name):
    import torch
    scn = _case(name, solver)
    g = scn.grid
    S = omp_state(g.mesh, g)
    P = oracle_params(scn.cfg)
    T = ST.TorchStep(g.mesh, scaling=scn.cfg.scaling, drytol=scn.cfg.dry_tolerance, bc=scn.cfg.boundary,
                     solver=solver)
    x = [torch.tensor(a) for a in (g.h, g.hu, g.hv)]
    b = torch.tensor(g.b)
    for step in range(4):
        dt = float(S.scal[1])
        S.steps(P, 1)
        x = list(T.step(*x, b, dt, step))
        for name_, a, ref in (("h", x[0], S.h), ("hu", x[1], S.hu), ("hv", x[2], S.hv)):
            a = a.numpy()
            assert np.isfinite(a).all(), (solver, step, name_)
            assert np.array_equal(a, ref), (solver, step, name_, int((a != ref).sum()))
