"""Raster autotuner for a rive_cuda context.

The raster's speed depends on the workload's shape: small tiles cut the
triangles each tile walks but raise the bin entries and the per-tile fixed
cost; more resident CTAs per SM hide latency but share the SM's issue slots
and L1. Every configuration gives the same image within the parity tolerance,
so the choice is free: this module times each candidate on the caller's own
work with CUDA events on the caller's stream and leaves the fastest set on the
context.
"""
from __future__ import annotations

from dataclasses import dataclass

import torch

# (tile size in pixels, resident raster CTAs per SM; 0 = as many as fit)
CANDIDATES = ((16, 0), (16, 4), (16, 3), (8, 0), (32, 0))


@dataclass
class Trial:
    tile_size: int
    ctas_per_sm: int
    ms: float


def time_config(ctx, run, tile_size, ctas_per_sm, stream, warmup=2, iters=5):
    """Mean device milliseconds of `run(stream)` under one raster config."""
    ctx.set_raster_config(tile_size, ctas_per_sm)
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            run(stream)
        stream.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(iters):
            run(stream)
        e1.record(stream)
        e1.synchronize()
    return e0.elapsed_time(e1) / iters


def autotune(ctx, run, candidates=CANDIDATES, stream=None, warmup=2, iters=5):
    """Times `run(stream)` (one frame or one batch, enqueued on `stream`) under
    each candidate and leaves the fastest configured on `ctx`.

    Returns (best Trial, all Trials). `run` must enqueue the same work each
    call; a CUDA graph built before the call keeps the configuration it was
    built with, so pass a `run` that builds nothing or rebuilds its graph.
    """
    stream = stream or torch.cuda.current_stream()
    trials = [Trial(t, c, time_config(ctx, run, t, c, stream, warmup, iters))
              for t, c in candidates]
    best = min(trials, key=lambda r: r.ms)
    ctx.set_raster_config(best.tile_size, best.ctas_per_sm)
    return best, trials
