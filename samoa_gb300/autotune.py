"""Autotuner of the step's tiling: segment length (cells per CTA pass) and
threads per CTA, timed on the device with CUDA events.

Tuning runs on a scratch context with the caller's mesh and state (the
caller's context keeps its state and step count), so it can run at any time,
e.g. after a remesh. A sample of the mesh is enough: the cost per cell of the
fused kernel does not depend on the mesh size once the GPU is full.
"""
import itertools

import numpy as np

from . import swe

DEFAULT_SEGMENTS = (256, 384, 448, 512, 640, 768, 1024)
DEFAULT_THREADS = (128, 256)
DEFAULT_STAGING = (1, 2)


def autotune(mesh, h, hu, hv, b, params, dt, segments=DEFAULT_SEGMENTS, threads=DEFAULT_THREADS, steps=4,
             device=0, staging=DEFAULT_STAGING, candidates=None):
    """Return ((segment_cells, block_threads, staging_depth), {setting: seconds per
    step}) for the fastest setting of segment length, block size and staging depth
    (every combination, or the given (segment_cells, block_threads, staging_depth)
    candidates, e.g. the best few of a search on a smaller sample)."""
    import torch
    ctx = swe.SweContext(device)
    results = {}
    try:
        ctx.set_params(params)
        ctx.upload_mesh(mesh)
        stream = torch.cuda.Stream(device=device)
        ctx.set_stream(stream.cuda_stream)
        settings = [(d, sg, t) for sg, t, d in candidates] if candidates else \
            list(itertools.product(staging, segments, threads))
        for depth, seg, thr in settings:
            try:
                ctx.set_staging(1)
                ctx.set_tiling(seg, thr)
                ctx.set_staging(depth)
            except swe._lib.SweError:
                continue
            ctx.upload_state(h, hu, hv, b)
            ctx.set_time(0.0, dt)
            ctx.traverse(1)  # warm-up
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            ctx.traverse(steps)
            e1.record(stream)
            e1.synchronize()
            ctx.synchronize()
            results[(seg, thr, depth)] = e0.elapsed_time(e1) * 1e-3 / steps
    finally:
        ctx.close()
    best = min(results, key=results.get)
    return best, results
