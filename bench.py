#!/usr/bin/env python
"""Throughput of the GB300 SWE time step: cell-updates/s and the HBM roofline.

Workload: synthetic ocean basin, 2^26 = 67,108,864 cells (reference depth 25),
uniform Sierpinski mesh, FP64, f-wave solver, outflow boundaries. One bench
step is one explicit Euler time step over the whole mesh (the reference's
``swe%euler%traverse(grid)``). The state (2.1 GB) is larger than L2, so no
flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

N > 1 runs N independent replicas (one per GPU, launched by torchrun); the
path does not shard across GPUs here ("replicas only"). ``--impl reference``
times the CPU implementation of the step (the project's OpenMP restatement of
the reference's FP64 step; the reference itself is Fortran and is not built)
on all host cores, on the whole workload, K steps in one call.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_CELL = 56  # read h, hu, hv, b + write h, hu, hv (FP64)
METRIC = "swe_cell_updates_per_s"
UNIT = "cell-updates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--log2-cells", type=int, default=26)
    ap.add_argument("--solver", default="fwave")
    ap.add_argument("--workload", default="basin", choices=["basin", "bowl"],
                    help="basin: the synthetic ocean basin (the headline); bowl: the wet/dry parabolic bowl, "
                         "half dry land (a parity case, for profiling the wet/dry paths and the solvers)")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-tune", action="store_true", help="skip the tiling autotuner (default tiling)")
    ap.add_argument("--no-adaptive", action="store_true")
    ap.add_argument("--adaptive-min-depth", type=int, default=12)
    ap.add_argument("--adaptive-max-depth", type=int, default=22)
    ap.add_argument("--adaptive-steps", type=int, default=500)
    ap.add_argument("--tune-log2-cells", type=int, default=22)
    ap.add_argument("--cpu-steps", type=int, default=20,
                    help="steps of the CPU baseline on the workload (20 x 2^26 cells: ~10 s on 16 Grace cores)")
    ap.add_argument("--segment-cells", type=int, default=0)
    ap.add_argument("--block-threads", type=int, default=0)
    ap.add_argument("--arith", default="strict", choices=["strict", "fma"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--ensemble-instances", type=int, default=512)
    ap.add_argument("--ensemble-steps", type=int, default=1000)
    ap.add_argument("--ensemble-bucket-steps", type=int, default=50,
                    help="steps of the per-size breakdown (batched and looped per log2-size bucket)")
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--adjoint-log2-cells", type=int, default=18)
    ap.add_argument("--adjoint-steps", type=int, default=2000)
    ap.add_argument("--adjoint-fd", type=int, default=16)
    ap.add_argument("--adjoint-fd-frozen", type=int, default=16,
                    help="directions of the branch-frozen finite-difference check of the adjoint")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-moving", action="store_true")
    ap.add_argument("--moving-log2-cells", type=int, default=22)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0}, "fallback"


def profile_figure(key):
    """A figure from the committed ncu summary of the step kernel, or None."""
    path = os.path.join(ROOT, "profiles", "swe_step_fwave_basin.md")
    try:
        with open(path) as f:
            for line in f:
                if line.strip().startswith(key + ":"):
                    return float(line.split(":", 1)[1].split()[0])
    except Exception:
        pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                p = [x.strip() for x in line.split(",")]
                if len(p) < 9:
                    continue
                try:
                    sm.append(float(p[1]))
                    smax = float(p[2])
                except ValueError:
                    continue
                for n, v in zip(names, p[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def host_cpu():
    """The host CPU's model name and logical core count (lscpu, else /proc/cpuinfo)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.split(":")[0].strip() in ("Model name", "Model"):
                model = line.split(":", 1)[1].strip()
                if not model.isdigit():
                    break
    except Exception:
        pass
    return {"model": model, "logical_cores": os.cpu_count()}


def oracle_params_for(cfg):
    from oracle import oracle as O
    from samoa_gb300 import swe
    return O.make_params(solver=swe.SOLVERS[cfg.flux_solver], bc=swe.BOUNDARIES[cfg.boundary],
                         dry_tolerance=cfg.dry_tolerance, courant=cfg.courant_number, scaling=cfg.scaling,
                         min_depth=cfg.i_min_depth, max_depth=cfg.i_max_depth)


def cpu_baseline(grid, cfg, steps, threads):
    """Time the OpenMP CPU step (the oracle's restatement of the reference step)
    on the bench workload itself: `steps` steps in one call, all host threads."""
    from oracle import oracle as O
    m = grid.mesh
    S = O.OmpState(m.depth, m.plotter, m.edge_cells, m.edge_local, m.bnd_cell, m.bnd_local, grid.h, grid.hu,
                   grid.hv, grid.b, grid.r_time, grid.r_dt)
    P = oracle_params_for(cfg)
    S.steps(P, 1, threads)  # warm-up
    t0 = time.perf_counter()
    S.steps(P, steps, threads)
    t = time.perf_counter() - t0
    return m.n_cells * steps / t, t


def basin_from_oracle(log2_cells, solver):
    """The basin workload on the oracle's own mesh (its walk of the Sierpinski
    grammar, oracle_mesh_uniform + oracle_mesh_edges), with the scenario's field
    generators evaluated on the oracle's cell centroids: the CPU arm loads no
    part of the GPU library."""
    from oracle import oracle as O
    from samoa_gb300 import scenarios, swe
    om = O.mesh_uniform(log2_cells - 1)
    c5, co = om["cells5"], om["coords"]
    cen = ((co[:, 0] + co[:, 1]) + co[:, 2]) / 3.0
    del om["coords"], co
    mesh = swe.Mesh(c5[:, 1].copy(), c5[:, 2].copy(), om["edge_cells"], om["edge_local"], om["bnd_cell"],
                    om["bnd_local"], cen)
    return scenarios.ocean_basin(log2_cells=log2_cells, solver=solver, mesh=mesh)


def run_reference(a, rank, world):
    if rank != 0:
        return 0
    from oracle import oracle as O
    threads = O.max_threads()
    scn = basin_from_oracle(a.log2_cells, a.solver)
    g = scn.grid
    m = g.mesh
    S = O.OmpState(m.depth, m.plotter, m.edge_cells, m.edge_local, m.bnd_cell, m.bnd_local, g.h, g.hu, g.hv, g.b,
                   g.r_time, g.r_dt)
    P = oracle_params_for(scn.cfg)
    S.steps(P, a.warmup, threads)
    t0 = time.perf_counter()
    S.steps(P, a.steps, threads)  # the K steps in one call, as the reference's run loop does
    t = time.perf_counter() - t0
    value = m.n_cells * a.steps / t
    sample = ("the whole workload: %d cells, %d steps in one call after %d warm-up steps, OpenMP C restatement "
              "of the reference step on the oracle's own mesh" % (m.n_cells, a.steps, a.warmup))
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
        "ms_per_step": 1000.0 * t / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": "ocean_basin_2^%d_cells_%s_fp64" % (a.log2_cells, a.solver), "cells": m.n_cells,
                   "solver": a.solver, "boundary": "outflow"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                         "host": host_cpu()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))
    return 0


def fp64_dgemm_tflops(torch):
    """Measured FP64 peak on this GPU: cuBLAS DGEMM 8192^3, best of 3."""
    n = 8192
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = max(best, 2.0 * n ** 3 / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    del a, b
    torch.cuda.empty_cache()
    return best


ENSEMBLE_TILINGS = [(256, 128), (384, 128), (512, 128), (512, 256)]
E2E_TILINGS = [(384, 128, 1), (384, 128, 2), (256, 128, 2), (512, 128, 2), (512, 256, 1), (512, 256, 2),
               (640, 256, 1), (768, 256, 1)]


def _time_batched(meshes, grids, cfgs, K, stream, device, tiling=None):
    """Seconds of K steps of the batched ensemble (one launch per step for all
    instances, replayed as a CUDA graph), after a warm-up replay."""
    import torch

    from samoa_gb300 import swe
    cat = lambda k: np.concatenate([getattr(g, k) for g in grids])
    batched = swe.SweEnsemble(device)
    try:
        if tiling:
            batched.set_tiling(*tiling)
        batched.upload_meshes(meshes)
        batched.set_params_list([c.params() for c in cfgs])
        batched.upload_state(cat("h"), cat("hu"), cat("hv"), cat("b"))
        batched.set_times([0.0] * len(grids), [g.r_dt for g in grids])
        batched.set_stream(stream.cuda_stream)
        batched.traverse_graph(K)  # capture + warm-up
        batched.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batched.traverse_graph(K)
        e1.record(stream)
        e1.synchronize()
        batched.synchronize()
        return e0.elapsed_time(e1) * 1e-3
    finally:
        batched.close()


def _time_looped(meshes, grids, cfgs, K, stream, device):
    """Seconds of K steps of the plain step launched per instance, one context per
    instance, all on one stream, after one warm-up step each."""
    import torch

    from samoa_gb300 import swe
    ctxs = []
    try:
        for m, g, c in zip(meshes, grids, cfgs):
            x = swe.SweContext(device)
            ctxs.append(x)
            x.set_params(c.params())
            x.upload_mesh(m)
            x.upload_state(g.h, g.hu, g.hv, g.b)
            x.set_time(0.0, g.r_dt)
            x.set_stream(stream.cuda_stream)
        for x in ctxs:
            x.traverse(1)  # warm-up
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(K):
            for x in ctxs:
                x.traverse(1)
        e1.record(stream)
        e1.synchronize()
        for x in ctxs:
            x.synchronize()
        return e0.elapsed_time(e1) * 1e-3
    finally:
        for x in ctxs:
            x.close()


def ensemble_compare(a, device):
    """Batched ensemble (one launch per step for all instances, replayed as a
    CUDA graph) against looping the plain step over the same instances (one
    context per instance, all on one stream), same GPU, same steps; then the
    same comparison per log2-size bucket of the instances."""
    import torch

    from samoa_gb300 import scenarios
    ens = scenarios.bowl_ensemble(n_instances=a.ensemble_instances, seed=4, device="cuda")
    cells = int(sum(m.n_cells for m in ens.meshes))
    K = a.ensemble_steps
    stream = torch.cuda.Stream(device=device)
    # the batched context's tiling: a short search over segment length x block size
    # (10 steps each, untimed in the result), as the plain step's autotuner does
    trial = {t: _time_batched(ens.meshes, ens.grids, ens.cfgs, 10, stream, device, tiling=t)
             for t in ENSEMBLE_TILINGS}
    best = min(trial, key=trial.get)
    t_batched = _time_batched(ens.meshes, ens.grids, ens.cfgs, K, stream, device, tiling=best)
    t_loop = _time_looped(ens.meshes, ens.grids, ens.cfgs, K, stream, device)
    v_b = cells * K / t_batched
    v_l = cells * K / t_loop
    buckets = {}
    Kb = a.ensemble_bucket_steps
    sizes = np.array([m.n_cells for m in ens.meshes])
    for k in sorted(set(int(x).bit_length() - 1 for x in sizes)):
        idx = [i for i in range(len(sizes)) if sizes[i] == 1 << k]
        sel = lambda xs: [xs[i] for i in idx]
        c = int(sizes[idx].sum())
        tb = _time_batched(sel(ens.meshes), sel(ens.grids), sel(ens.cfgs), Kb, stream, device, tiling=best)
        tl = _time_looped(sel(ens.meshes), sel(ens.grids), sel(ens.cfgs), Kb, stream, device)
        buckets["2^%d" % k] = {"instances": len(idx), "cells": c, "batched": c * Kb / tb, "looped": c * Kb / tl,
                               "speedup": tl / tb, "looped_ms_per_step": 1e3 * tl / Kb,
                               "batched_ms_per_step": 1e3 * tb / Kb}
    return {"instances": len(ens.grids), "cells": cells, "steps": K, "batched": v_b, "looped": v_l,
            "speedup": v_b / v_l, "unit": UNIT, "batched_ms_per_step": 1e3 * t_batched / K,
            "batched_tiling": list(best), "tiling_trials_ms_per_step": {"%dx%d" % k: 1e2 * v for k, v in trial.items()},
            "looped_ms_per_step": 1e3 * t_loop / K, "per_size": {"steps": Kb, "buckets": buckets},
            "note": "bowl ensemble, 2^12..2^20 cells per instance, f-wave, own dt per instance; batched = one "
                    "launch per step for all instances replayed as a CUDA graph; looped = the plain step launched "
                    "per instance on one stream; per_size: the same comparison for the instances of each size "
                    "alone"}


def rest_edge_fraction(mesh, h, hu, hv, b, drytol):
    """The share of inner edges whose two cells hold water at rest under one
    surface (both momenta +-0 on both sides, both depths above the dry
    tolerance, ((bR + dR) - bL) - dL == 0): the edges the f-wave step resolves
    by its exact lake-at-rest path. Host numpy on the state after the run."""
    ec = mesh.edge_cells
    frac, n = 0, len(ec)
    for s in range(0, n, 1 << 24):
        e = ec[s:s + (1 << 24)]
        L, R = e[:, 0], e[:, 1]
        dL, dR = h[L] - b[L], h[R] - b[R]
        still = (hu[L] == 0) & (hv[L] == 0) & (hu[R] == 0) & (hv[R] == 0)
        wet = (dL > drytol) & (dR > drytol)
        surf = ((b[R] + dR) - b[L]) - dL
        frac += int(np.count_nonzero(still & wet & (surf == 0)))
    return frac / max(n, 1)


def moving_water(a, device):
    """The step's rate where the water moves: the wet/dry parabolic bowl with a
    2 m Gaussian bump (2^22 cells, f-wave, 20 steps after 3 warm-up steps), where
    few edges are at rest, against the headline workload's rate."""
    import torch

    from samoa_gb300 import scenarios, swe
    scn = scenarios.parabolic_bowl(log2_cells=a.moving_log2_cells, solver=a.solver, amplitude=2.0, sigma=0.08)
    g = scn.grid
    ctx = swe.SweContext(device)
    try:
        ctx.set_params(scn.cfg.params())
        ctx.upload_mesh(g.mesh)
        ctx.upload_state(g.h, g.hu, g.hv, g.b)
        ctx.set_time(0.0, g.r_dt)
        stream = torch.cuda.Stream(device=device)
        ctx.set_stream(stream.cuda_stream)
        ctx.traverse(3)
        ctx.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        ctx.traverse(20)
        e1.record(stream)
        e1.synchronize()
        ctx.synchronize()
        t = e0.elapsed_time(e1) * 1e-3
        h, hu, hv, b = ctx.download_state()
        rest = rest_edge_fraction(g.mesh, h, hu, hv, b, scn.cfg.dry_tolerance)
    finally:
        ctx.close()
    return {"workload": "parabolic_bowl_2^%d_cells_%s_fp64" % (a.moving_log2_cells, a.solver),
            "value": g.mesh.n_cells * 20 / t, "unit": UNIT, "steps": 20, "rest_edge_fraction": rest,
            "note": "half of the bowl is dry land, the wet half moves"}


def adaptive_compare(a, device):
    """The adaptive wet/dry bowl (augmented Riemann, dry tolerance 1e-3) with a
    host remesh before every step (nadapt 1): device time of the steps against
    host time of the remeshes (swe_mesh_adapt + swe_mesh_build + upload)."""
    from samoa_gb300 import scenarios, swe
    t0 = time.perf_counter()
    scn = scenarios.adaptive_bowl(min_depth=a.adaptive_min_depth, max_depth=a.adaptive_max_depth)
    t_init = time.perf_counter() - t0
    g = scn.grid
    (mesh, *_), st = swe.run_adaptive(scn.cfg, g.mesh, g.h, g.hu, g.hv, g.b, g.r_dt, a.adaptive_steps,
                                      adapt_every=1, bathymetry=scenarios.bowl_bathymetry, device=device)
    return {"workload": "adaptive_bowl_aug_riemann_dmin%d_dmax%d" % (a.adaptive_min_depth, a.adaptive_max_depth),
            "steps": st["steps"], "cells_first": st["cells"][0], "cells_last": st["cells"][-1],
            "apriori_refinement_s": t_init, "step_cell_updates_per_s": st["cell_updates"] / st["step_s"],
            "remesh_s_per_step": st["remesh_s"] / max(1, st["remeshes"]),
            "remesh_parts_s_per_step": {k: st[k + "_s"] / max(1, st["remeshes"]) for k in ("download", "adapt", "upload")},
            "step_s_per_step": st["step_s"] / st["steps"],
            "end_to_end_cell_updates_per_s": st["cell_updates"] / (st["step_s"] + st["remesh_s"]),
            "note": "remesh before every step from the previous step's flags (host C++: conformity, "
                    "refine/coarsen, order-0 transfer, edge streams), then upload; the step itself on the GPU"}


def adjoint_compare(a, device):
    """Gauge-misfit gradient through the adjoint against the forward run it
    differentiates: 2^18 cells, 2,000 steps, 64 snapshots, f-wave, frozen dt;
    the gradient is checked by central differences in seeded random directions."""
    from samoa_gb300 import adjoint, scenarios
    case = scenarios.adjoint_case(log2_cells=a.adjoint_log2_cells, steps=a.adjoint_steps, n_gauges=32, seed=5,
                                  device=device)
    P = adjoint.GaugeProblem(case["mesh"], case["params"], case["gauges"], case["obs"], case["dts"], snapshots=64,
                             device=device)
    try:
        P.objective(case["h0"], case["b"], record=False)  # warm-up
        t0 = time.perf_counter()
        J = P.objective(case["h0"], case["b"], record=False)
        t_fwd = time.perf_counter() - t0
        P.gradient(case["h0"], case["b"])  # warm-up
        P.stats = {"forward_steps": 0, "adjoint_steps": 0}
        t0 = time.perf_counter()
        J2, gh, gb = P.gradient(case["h0"], case["b"])
        t_grad = time.perf_counter() - t0
        stats = dict(P.stats)
        gh, gb = gh.cpu().numpy(), gb.cpu().numpy()
        rng = np.random.default_rng(16)
        # directions supported off the flat -20 m shelf: there neighbouring depths
        # are equal, every edge sits on the Einfeldt min/max kink, and central
        # differences straddle it
        deep = case["b"] < -100.0
        errs = {"h0": [], "b": []}
        nerr = []  # |fd - ad| / (|g| |d|): the error against the directional scale of the gradient
        for key, n_dir in (("h0", a.adjoint_fd), ("b", max(1, a.adjoint_fd // 4) if a.adjoint_fd else 0)):
            for k in range(n_dir):
                d = rng.normal(size=gh.shape) * deep
                if key == "h0":
                    eps = 1e-6 * float(np.abs(case["h0"]).max())
                    Jp = P.objective(case["h0"] + eps * d, case["b"], record=False)
                    Jm = P.objective(case["h0"] - eps * d, case["b"], record=False)
                    ad = float(gh @ d)
                else:
                    eps = 1e-6 * float(np.abs(case["b"]).max())
                    Jp = P.objective(case["h0"], case["b"] + eps * d, record=False)
                    Jm = P.objective(case["h0"], case["b"] - eps * d, record=False)
                    ad = float(gb @ d)
                errs[key].append(abs((Jp - Jm) / (2 * eps) - ad) / max(abs(ad), 1e-300))
                if key == "h0":
                    nerr.append(abs((Jp - Jm) / (2 * eps) - ad) / max(np.linalg.norm(gh) * np.linalg.norm(d), 1e-300))
        # the same check on the branch-frozen J (every decision of the unperturbed run
        # replayed): 4-point central differences, no kink crossed
        P.objective_frozen(case["h0"], case["b"], record=True)
        ferrs = []
        for k in range(a.adjoint_fd_frozen):
            d = rng.normal(size=gh.shape)
            eps = 1e-4 * float(np.abs(case["h0"]).max())  # smooth J: the round-off of J sets the step
            Jf = lambda s_: P.objective_frozen(case["h0"] + s_ * eps * d, case["b"], record=False)
            fd = (8.0 * (Jf(1) - Jf(-1)) - (Jf(2) - Jf(-2))) / (12.0 * eps)
            ad = float(gh @ d)
            ferrs.append(abs(fd - ad) / max(abs(ad), 1e-300))
        fb, fbr = None, []
        if a.adjoint_fd_frozen:
            d = gb / np.linalg.norm(gb)
            eps = 1e-4 * float(np.abs(case["b"]).max())
            Jf = lambda s_: P.objective_frozen(case["h0"], case["b"] + s_ * eps * d, record=False)
            fd = (8.0 * (Jf(1) - Jf(-1)) - (Jf(2) - Jf(-2))) / (12.0 * eps)
            fb = abs(fd - float(gb @ d)) / abs(float(gb @ d))
            # random directions of b: the directional derivative can be tiny (the flat shelf),
            # so the error is taken against the gradient's scale
            for k in range(4):
                d = rng.normal(size=gb.shape)
                Jf = lambda s_: P.objective_frozen(case["h0"], case["b"] + s_ * eps * d, record=False)
                fd = (8.0 * (Jf(1) - Jf(-1)) - (Jf(2) - Jf(-2))) / (12.0 * eps)
                fbr.append(abs(fd - float(gb @ d)) / (np.linalg.norm(gb) * np.linalg.norm(d)))
        t_step, t_adj = adjoint.time_steps(P, case["h0"], case["b"], 50)
    finally:
        P.close()
    all_states = adjoint_all_states(a, case, device, t_fwd, J)
    windowed = adjoint_windowed(a, case, device)
    try:
        moving_fd = adjoint_moving_fd(device)
    except Exception as exc:
        moving_fd = {"error": repr(exc)[:300]}
    n = case["mesh"].n_cells
    return {"cells": n, "steps": a.adjoint_steps, "snapshots": 64, "J": J, "forward_s": t_fwd, "gradient_s": t_grad,
            "gradient_over_forward": t_grad / t_fwd, "forward_steps_in_gradient": stats["forward_steps"],
            "adjoint_steps": stats["adjoint_steps"], "fd_directions_h0": len(errs["h0"]),
            "fd_max_rel_err_h0": max(errs["h0"], default=None),
            "fd_median_rel_err_h0": float(np.median(errs["h0"])) if errs["h0"] else None,
            "fd_directions_h0_within_1e-6": int(sum(e <= 1e-6 for e in errs["h0"])),
            "fd_max_err_over_grad_norm_h0": max(nerr, default=None),
            "fd_directions_b": len(errs["b"]), "fd_max_rel_err_b_unfrozen": max(errs["b"], default=None),
            "fd_frozen_directions_h0": len(ferrs), "fd_frozen_max_rel_err_h0": max(ferrs, default=None),
            "fd_frozen_rel_err_b_along_gradient": fb, "fd_frozen_directions_b": len(fbr),
            "fd_frozen_max_err_over_grad_norm_b": max(fbr, default=None),
            "forward_step_ms": 1e3 * t_step, "adjoint_step_ms": 1e3 * t_adj, "adjoint_step_over_forward_step": t_adj / t_step,
            "windowed": windowed, "all_states": all_states, "fd_moving_water": moving_fd,
            "note": "gradient_s = one checkpointed sweep (its first descent is the forward run; recomputation "
                    "included); J(h0, b) is the squared misfit at 32 gauges; dt frozen, FD with the same dts, "
                    "eps = 1e-6 relative, seeded N(0,1) directions on the cells deeper than 100 m. J is piecewise "
                    "smooth: in the nearly still basin the f-wave's middle wave speed 0.5 (s1 + s2) sits near 0, and "
                    "its sign sends the shear wave to the left or the right cell, so perturbations flip branches and "
                    "J jumps slightly; the per-direction error is branch-limited (measured: not monotone in eps, "
                    "no better with a 4-point stencil), the error against |g| |d| stays small; fd_frozen_*: the same "
                    "check on the branch-frozen J (swe_traverse_frozen replays every decision of the unperturbed "
                    "run), 4-point stencil, eps = 1e-4 relative, seeded N(0,1) directions over all cells, where it "
                    "is not branch-limited; b along its gradient and in 4 random directions (error against "
                    "|g| |d|: the shelf is flat, so many directional derivatives are tiny). Perturbing b "
                    "reorders neighbouring depths at rest and so crosses the Einfeldt min/max kinks over 2,000 "
                    "steps, so plain FD in b is kink-limited"}


def adjoint_all_states(a, case, device, t_fwd, J):
    """The same gradient with a slot for every step's state (2,000 x 24 B x 2^18
    cells = 12.6 GB of HBM) instead of the configuration's 64: the first descent
    stores every state and no step is recomputed, which separates the cost of
    the 64-slot budget from the cost of the reverse steps themselves."""
    from samoa_gb300 import adjoint
    P = adjoint.GaugeProblem(case["mesh"], case["params"], case["gauges"], case["obs"], case["dts"],
                             snapshots=a.adjoint_steps, device=device)
    try:
        P.gradient(case["h0"], case["b"])  # warm-up
        P.stats = {"forward_steps": 0, "adjoint_steps": 0}
        t0 = time.perf_counter()
        Jg, _, _ = P.gradient(case["h0"], case["b"])
        t_grad = time.perf_counter() - t0
        stats = dict(P.stats)
    finally:
        P.close()
    return {"snapshots": a.adjoint_steps, "gradient_s": t_grad, "gradient_over_forward": t_grad / t_fwd,
            "forward_steps_in_gradient": stats["forward_steps"], "J_rel_diff": abs(Jg - J) / abs(J),
            "note": "not the configuration (64 stored states): every state kept, no recomputation"}


def adjoint_moving_fd(device, steps=100, n_dir=6):
    """Plain central differences of J where the water moves everywhere: the
    current basin (2^12 cells, a uniform (2, 1) m/s current over 80-120 m of
    depth, 100 steps, frozen dt), where no wave speed sits at 0 and nothing is
    dry, so J has no jumps. Error against the adjoint gradient in seeded
    directions of the initial surface (momenta held)."""
    from samoa_gb300 import adjoint, scenarios, swe
    scn = scenarios.current_basin(log2_cells=12)
    g = scn.grid
    ctx = swe.SweContext(device)
    try:
        ctx.set_params(scn.cfg.params())
        ctx.upload_mesh(g.mesh)
        ctx.upload_state(g.h, g.hu, g.hv, g.b)
        ctx.set_time(0.0, g.r_dt)
        ctx.traverse(1)
        _, dt, _ = ctx.get_time()
    finally:
        ctx.close()
    rng = np.random.default_rng(8)
    gauges = np.sort(rng.choice(g.mesh.n_cells, 12, replace=False))
    obs = rng.normal(0.0, 0.05, (steps, 12))
    P = adjoint.GaugeProblem(g.mesh, scn.cfg.params(), gauges, obs, np.full(steps, 0.8 * dt), snapshots=8,
                             device=device)
    try:
        _, gh, _ = P.gradient_python(g.h, g.b, g.hu, g.hv)
        gh = gh.cpu().numpy()
        errs = []
        for _ in range(n_dir):
            d = rng.normal(size=g.mesh.n_cells)
            eps = 1e-5 * np.abs(g.h).max()
            Jp = P.objective(g.h + eps * d, g.b, record=False, hu0=g.hu, hv0=g.hv)
            Jm = P.objective(g.h - eps * d, g.b, record=False, hu0=g.hu, hv0=g.hv)
            ad = float(gh @ d)
            errs.append(abs((Jp - Jm) / (2 * eps) - ad) / max(abs(ad), 1e-300))
    finally:
        P.close()
    return {"workload": "current_basin_2^12_cells_fwave", "steps": steps, "directions_h0": n_dir,
            "max_rel_err_h0": max(errs), "note": "plain central differences (eps 1e-5 relative), no branch freezing"}


def adjoint_windowed(a, case, device):
    """The same problem with the adaptive mesh frozen per 50-step window: after
    each window the mesh adapts from its last step's flags between depths d - 2
    and d + 1 (the uniform depth d in the first window), state and bathymetry
    carried over by the order-0 transfer, gauges re-located; the gradient chains
    the windows' checkpointed adjoints through the transfers' adjoints. Checked by
    central differences with the mesh sequence frozen."""
    import copy

    from samoa_gb300 import adjoint
    mesh = case["mesh"]
    cfg = copy.copy(case["cfg"])
    d = int(mesh.depth[0])
    cfg.i_min_depth, cfg.i_max_depth = d - 2, d + 1
    pts = cfg.scaling * mesh.centroids[case["gauges"]] + np.asarray(cfg.offset, np.float64)
    W = adjoint.WindowedGaugeProblem(mesh, cfg, pts, case["obs"], case["dts"], window=50, snapshots=64,
                                     device=device)
    W.objective(case["h0"], case["b"])  # fixes the mesh sequence (and warms up)
    t0 = time.perf_counter()
    J = W.objective(case["h0"], case["b"])
    t_fwd = time.perf_counter() - t0
    W.gradient(case["h0"], case["b"])  # warm-up: a first call on a fresh box pays several seconds of first use
    t0 = time.perf_counter()
    Jg, gh, gb = W.gradient(case["h0"], case["b"])
    t_grad = time.perf_counter() - t0
    rng = np.random.default_rng(17)
    deep = case["b"] < -100.0
    errs = []
    for _ in range(4):
        dd = rng.normal(size=mesh.n_cells) * deep
        eps = 1e-6 * float(np.abs(case["h0"]).max())
        fd = (W.objective(case["h0"] + eps * dd, case["b"]) - W.objective(case["h0"] - eps * dd, case["b"])) / (2 * eps)
        ad = float(gh @ dd)
        errs.append(abs(fd - ad) / max(abs(ad), 1e-300))
    # branch-frozen J: every window's decisions recorded once, then replayed
    ferrs, fb, fbr = [], None, []
    if a.adjoint_fd_frozen:
        Jrec = W.objective_frozen(case["h0"], case["b"], record=True)
        assert Jrec == J, (Jrec, J)
        for _ in range(a.adjoint_fd_frozen):
            dd = rng.normal(size=mesh.n_cells)
            eps = 1e-4 * float(np.abs(case["h0"]).max())
            Jf = lambda s_: W.objective_frozen(case["h0"] + s_ * eps * dd, case["b"], record=False)
            fd = (8.0 * (Jf(1) - Jf(-1)) - (Jf(2) - Jf(-2))) / (12.0 * eps)
            ad = float(gh @ dd)
            ferrs.append(abs(fd - ad) / max(abs(ad), 1e-300))
        eps = 1e-4 * float(np.abs(case["b"]).max())
        for k in range(5):  # b along its gradient, then random directions (error against |g| |d|)
            dd = gb / np.linalg.norm(gb) if k == 0 else rng.normal(size=mesh.n_cells)
            Jf = lambda s_: W.objective_frozen(case["h0"], case["b"] + s_ * eps * dd, record=False)
            fd = (8.0 * (Jf(1) - Jf(-1)) - (Jf(2) - Jf(-2))) / (12.0 * eps)
            ad = float(gb @ dd)
            if k == 0:
                fb = abs(fd - ad) / abs(ad)
            else:
                fbr.append(abs(fd - ad) / (np.linalg.norm(gb) * np.linalg.norm(dd)))
    cells = W.stats["cells"]
    return {"window": 50, "windows": len(cells), "depths": [d - 2, d + 1], "cells_first": cells[0],
            "cells_min": min(cells), "cells_max": max(cells), "J": J, "forward_s": t_fwd, "gradient_s": t_grad,
            "gradient_over_forward": t_grad / t_fwd, "fd_directions_h0": len(errs), "fd_max_rel_err_h0": max(errs),
            "fd_frozen_directions_h0": len(ferrs), "fd_frozen_max_rel_err_h0": max(ferrs, default=None),
            "fd_frozen_rel_err_b_along_gradient": fb, "fd_frozen_directions_b": len(fbr),
            "fd_frozen_max_err_over_grad_norm_b": max(fbr, default=None),
            "note": "gradient_s and forward_s include the host work between windows (mesh upload, transfer, "
                    "gauge location); the forward run that fixes the mesh sequence is not timed; fd_*: plain "
                    "central differences (eps 1e-6 relative, deep cells), branch-limited like the uniform mesh's; "
                    "fd_frozen_*: 4-point differences of the branch-frozen J (eps 1e-4 relative, all cells)"}


def run_gpu(a, rank, world, local):
    import torch
    import torch.distributed as dist

    from samoa_gb300 import build as lib_build
    lib_build.build()
    from samoa_gb300 import scenarios, swe

    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    if a.workload == "bowl":
        scn = scenarios.parabolic_bowl(log2_cells=a.log2_cells, solver=a.solver, amplitude=2.0, sigma=0.08)
    else:
        scn = scenarios.ocean_basin(log2_cells=a.log2_cells, solver=a.solver, device="cuda")
    g = scn.grid
    n = g.mesh.n_cells
    ctx = swe.SweContext(local)
    ctx.set_params(scn.cfg.params())
    ctx.set_arith(a.arith)
    tuning = None
    if a.segment_cells or a.block_threads:
        ctx.set_tiling(a.segment_cells, a.block_threads)
    elif not a.no_tune:  # the autotuner on a sample of the same basin (not timed)
        from samoa_gb300 import autotune
        sample = scenarios.ocean_basin(log2_cells=min(a.tune_log2_cells, a.log2_cells), solver=a.solver,
                                       device="cuda")
        sg = sample.grid
        best, res = autotune.autotune(sg.mesh, sg.h, sg.hu, sg.hv, sg.b, sample.cfg.params(), sg.r_dt, device=local)
        tuning = {"sample_cells": sg.mesh.n_cells, "sample_best": list(best),
                  "ms_per_step": {"%dx%d/s%d" % k: round(v * 1e3, 4) for k, v in sorted(res.items())}}
        del sample, sg
        if a.tune_log2_cells < a.log2_cells:
            # the sample's best few, timed again on the workload itself: tail effects differ
            # between sizes, and near-ties on the sample need not be ties on the workload
            top = sorted(res, key=res.get)[:4]
            best, res2 = autotune.autotune(g.mesh, g.h, g.hu, g.hv, g.b, scn.cfg.params(), g.r_dt, device=local,
                                           candidates=top)
            tuning["workload_ms_per_step"] = {"%dx%d/s%d" % k: round(v * 1e3, 4) for k, v in sorted(res2.items())}
        tuning["best"] = list(best)
        ctx.set_staging(1)
        ctx.set_tiling(best[0], best[1])
        ctx.set_staging(best[2])
    ctx.upload_mesh(g.mesh)
    ctx.upload_state(g.h, g.hu, g.hv, g.b)
    ctx.set_time(g.r_time, g.r_dt)
    stream = torch.cuda.Stream(device=local)
    ctx.set_stream(stream.cuda_stream)
    tiling = ctx.get_tiling()
    counts = ctx.task_counts()

    # warm-up
    ctx.traverse(a.warmup)
    ctx.synchronize()

    # timed region: K steps, CUDA events on the launching stream
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.traverse(a.steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = e0.elapsed_time(e1)
    ctx.synchronize()  # raises if a kernel reported an error
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
        dist.barrier()
    sim_time, dt, _ = ctx.get_time()
    value = n * a.steps * world / (ms * 1e-3)
    hst = ctx.download_state()
    rest_frac = rest_edge_fraction(g.mesh, *hst, scn.cfg.dry_tolerance) if a.solver == "fwave" else None
    del hst

    # end to end through the public API with host buffers. Headline: swe_step_host,
    # the step reading the state from pinned host memory and writing the new state
    # and the flags back to pinned host memory inside the kernel (over the
    # coherent CPU-GPU link); every step completes (synchronised) before the next.
    # Also reported: the upload / traverse / download round trip with copies.
    e2e = None
    if not a.no_e2e:
        hs = [torch.from_numpy(np.ascontiguousarray(x)).pin_memory() for x in ctx.download_state()]
        cur, hb = hs[:3], hs[3]
        nxt = [torch.empty(n, dtype=torch.float64).pin_memory() for _ in range(3)]
        hflags = torch.zeros(n, dtype=torch.int8).pin_memory()
        ctx.step_host(*cur, hb, *nxt, hflags)  # warm-up
        ctx.synchronize()
        cur, nxt = nxt, cur
        # the host-memory step's own tiling: its loads wait on the CPU-GPU link rather
        # than on HBM, so a short search (3 steps each, untimed in the result) over
        # segment length, block size and staging depth picks it
        e2e_trials = {}
        if not (a.segment_cells or a.block_threads):
            for seg, blk, st in E2E_TILINGS:
                try:
                    ctx.set_staging(1)
                    ctx.set_tiling(seg, blk)
                    ctx.set_staging(st)
                except Exception:
                    continue
                ctx.step_host(*cur, None, *nxt, hflags)
                ctx.synchronize()
                t0 = time.perf_counter()
                for _ in range(3):
                    ctx.step_host(*cur, None, *nxt, hflags)
                    ctx.synchronize()
                e2e_trials[(seg, blk, st)] = (time.perf_counter() - t0) / 3
            if e2e_trials:
                seg, blk, st = min(e2e_trials, key=e2e_trials.get)
                ctx.set_staging(1)
                ctx.set_tiling(seg, blk)
                ctx.set_staging(st)
        if world > 1:
            dist.barrier()
        # b is the bathymetry: a host uploads it with the state after each remesh and
        # steps with b = NULL (the device copy); h, hu, hv cross the link every step
        t0 = time.perf_counter()
        for _ in range(a.e2e_steps):
            ctx.step_host(*cur, None, *nxt, hflags)
            ctx.synchronize()
            cur, nxt = nxt, cur
        te = time.perf_counter() - t0
        # the same with b read from host memory every step as well
        t0 = time.perf_counter()
        for _ in range(a.e2e_steps):
            ctx.step_host(*cur, hb, *nxt, hflags)
            ctx.synchronize()
            cur, nxt = nxt, cur
        tb = time.perf_counter() - t0
        hh, hu, hv = (t.numpy() for t in cur)
        flags = hflags.numpy()
        ctx.upload_state(hh, hu, hv, hb.numpy())
        ctx.synchronize()
        t0 = time.perf_counter()
        for _ in range(a.e2e_steps):
            ctx.upload_state(hh, hu, hv, hb.numpy())
            ctx.traverse(1)
            ctx.download_state([hh, hu, hv, hb.numpy()])
            ctx.refinements(flags)
        tc = time.perf_counter() - t0
        if world > 1:
            t = torch.tensor([te, tc, tb], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            te, tc, tb = (float(x) for x in t.tolist())
        e2e = {"value": n * a.e2e_steps * world / te, "unit": UNIT, "h2d_bytes_per_step": 24 * n,
               "tiling": list(min(e2e_trials, key=e2e_trials.get)) if e2e_trials else None,
               "tiling_trials_ms_per_step": {"%dx%d/s%d" % k: round(v * 1e3, 3) for k, v in e2e_trials.items()},
               "d2h_bytes_per_step": 24 * n + n, "steps": a.e2e_steps, "api": "swe_step_host",
               "note": "every step reads h, hu, hv from pinned host memory and writes h, hu, hv and the "
                       "refinement flags to pinned host memory inside the step kernel, then synchronises; b, "
                       "the bathymetry, stays on the device from the state upload (swe_step_host with b = NULL)",
               "b_from_host": {"value": n * a.e2e_steps * world / tb, "h2d_bytes_per_step": 32 * n,
                               "note": "the same with b read from pinned host memory every step"},
               "copy_round_trip": {"value": n * a.e2e_steps * world / tc, "h2d_bytes_per_step": 32 * n,
                                   "d2h_bytes_per_step": 32 * n + n + 40,
                                   "api": "swe_state_upload + swe_traverse + swe_state_download + "
                                          "swe_get_refinements"}}

    peaks, peak_kind = measured_peaks()
    peak = float(peaks.get("hbm_gbs", 6800.0))
    achieved = BYTES_PER_CELL * n / (ms * 1e-3 / a.steps) / 1e9
    traffic_per_cell = profile_figure("dram_bytes_per_cell")
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic_per_cell * n if traffic_per_cell else None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (%s)" % peak_kind,
                "kernels": "step_kernel, after cross_edges_kernel for the edges between two segments; "
                           "achieved over the time of both per step",
                "algorithmic_bytes_per_cell": BYTES_PER_CELL}

    out = None
    if rank == 0:
        fp64 = fp64_dgemm_tflops(torch)
        fp64_util = profile_figure("fp64_pipe_active_pct")
        fp64_per_cell = profile_figure("fp64_instr_per_cell")
        cpu = None
        if world == 1 and not a.no_cpu:
            from oracle import oracle as O
            threads = O.max_threads()
            v, t = cpu_baseline(g, scn.cfg, a.cpu_steps, threads)
            cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "host": host_cpu(),
                   "sample": "the whole workload (%d cells), %d steps in one call (%.1f s), OpenMP C restatement "
                             "of the reference step" % (n, a.cpu_steps, t)}
        ensemble = None
        if world == 1 and not a.no_ensemble:
            try:
                ensemble = ensemble_compare(a, local)
            except Exception as exc:  # reported, never hides the headline number
                ensemble = {"error": repr(exc)[:300]}
        adaptive = None
        if world == 1 and not a.no_adaptive:
            try:
                adaptive = adaptive_compare(a, local)
            except Exception as exc:
                adaptive = {"error": repr(exc)[:300]}
        moving = None
        if world == 1 and a.solver == "fwave" and not a.no_moving:
            try:
                moving = moving_water(a, local)
            except Exception as exc:
                moving = {"error": repr(exc)[:300]}
        adj = None
        if world == 1 and not a.no_adjoint:
            try:
                adj = adjoint_compare(a, local)
            except Exception as exc:
                adj = {"error": repr(exc)[:300]}
        out = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": ms / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": ("ocean_basin_2^%d_cells_%s_fp64" if a.workload == "basin" else
                                    "parabolic_bowl_2^%d_cells_%s_fp64") % (a.log2_cells, a.solver), "cells": n,
                       "solver": a.solver, "boundary": "outflow", "segment_cells": tiling[0],
                       "block_threads": tiling[1], "staging_depth": tuning["best"][2] if tuning else 1,
                       "arith": a.arith, "autotune": tuning, "cross_segment_edges": counts["cross_edges"],
                       "l2": "inputs larger than L2 (2.1 GB state)",
                       "parallelism": "replicas" if world > 1 else "single"},
            "roofline": roofline,
            "fp64": {"dgemm_tflops_measured": fp64, "fp64_pipe_active_pct_ncu": fp64_util,
                     "note": "the step is FP64-issue bound on GB300; see the ncu summary in profiles/"},
            # the bound that sets the pace: FP64 instructions per cell (ncu) x cells/s against the FP64
            # instruction rate of the measured DGEMM (one DFMA = 2 flops)
            "fp64_roofline": None if not (fp64 and fp64_per_cell) else {
                "bound": "fp64", "achieved": value * fp64_per_cell / 1e9,
                "peak": fp64 * 1e3 / 2.0, "unit": "G FP64 instructions/s",
                "frac": value * fp64_per_cell / 1e9 / (fp64 * 1e3 / 2.0),
                "instr_per_cell": fp64_per_cell,
                "source": "instr_per_cell from the ncu summary in profiles/, peak from the DGEMM measured above"},
            "cpu_baseline": cpu,
            "e2e": e2e,
            "rest_edge_fraction": rest_frac,
            "moving_water": moving,
            "ensemble": ensemble,
            "adjoint": adj,
            "adaptive": adaptive,
            "gpu_launches": a.steps * counts["launches_per_step"],
            "clocks": clk,
            "sim": {"time": sim_time, "dt": dt},
        }
        print(json.dumps(out))
    ctx.close()
    if world > 1:
        dist.destroy_process_group()
    return 0


def main():
    a = parse()
    rank, world, local = dist_env()
    if a.impl == "reference":
        return run_reference(a, rank, world)
    return run_gpu(a, rank, world, local)


if __name__ == "__main__":
    sys.exit(main())
