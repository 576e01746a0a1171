"""Raster autotuner for a rive_cuda context.

The flush's speed depends on the workload's shape: small tiles cut the
triangles each tile walks but raise the bin entries and the per-tile fixed
cost; more resident raster CTAs per SM hide latency but share the SM's issue
slots and L1; interior tiles as winding records pay on large filled shapes
and cost extra passes elsewhere. Every configuration gives the same image (bit
for bit for the winding records, within the parity tolerance across tile
sizes), so the choice is free: this module times each candidate on the
caller's own work with CUDA events on the caller's stream and leaves the
fastest set on the context.

The search space is tile size {8, 16, 32} x resident raster CTAs per SM
{1, 2, 4, as many as fit} x winding records {off, on}, and for 16-pixel
tiles the raster schedule {one CTA per tile, persistent work queue}; 32-pixel
tiles run one 1,024-thread CTA per SM at most, so only their "as many as fit"
entry differs.
"""
from __future__ import annotations

from dataclasses import dataclass

import torch

TILES = (8, 16, 32)
CTAS_PER_SM = (1, 2, 4, 0)  # 0 = as many as fit
WINDING = (False, True)


def _candidates():
    out = []
    for w in WINDING:
        for t in TILES:
            for c in (CTAS_PER_SM if t != 32 else (0,)):
                for q in ((False, True) if t == 16 else (False,)):
                    out.append((t, c, w, q))
    return tuple(out)


# (tile size in pixels, resident raster CTAs per SM or 0, winding records,
# work-queue raster)
CANDIDATES = _candidates()


@dataclass
class Trial:
    tile_size: int
    ctas_per_sm: int
    winding: bool
    queue: bool
    ms: float


def apply(ctx, tile_size, ctas_per_sm, winding, queue=False):
    ctx.set_raster_config(tile_size, ctas_per_sm)
    ctx.set_winding_tiles(winding)
    ctx.set_raster_queue(queue)


def time_config(ctx, run, tile_size, ctas_per_sm, winding, stream, warmup=2, iters=5,
                queue=False):
    """Mean device milliseconds of `run(stream)` under one configuration."""
    apply(ctx, tile_size, ctas_per_sm, winding, queue)
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
    each candidate (tile size, CTAs per SM, winding records, queue) and leaves the
    fastest configured on `ctx`.

    Returns (best Trial, all Trials). `run` must enqueue the same work each
    call; a CUDA graph built before the call keeps the configuration it was
    built with, so pass a `run` that builds nothing or rebuilds its graph.
    """
    stream = stream or torch.cuda.current_stream()
    trials = []
    for cand in candidates:
        t, c = cand[0], cand[1]
        w = cand[2] if len(cand) > 2 else False
        q = cand[3] if len(cand) > 3 else False
        trials.append(Trial(t, c, w, q, time_config(ctx, run, t, c, w, stream, warmup, iters, q)))
    best = min(trials, key=lambda r: r.ms)
    apply(ctx, best.tile_size, best.ctas_per_sm, best.winding, best.queue)
    return best, trials
