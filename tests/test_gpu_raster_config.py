"""Raster configurations (rive_cuda_set_raster_config): every tile size and
CTAs-per-SM limit must meet the same image bar against the oracle as the
default, in single flushes, in a batch and in a CUDA graph, and the
autotuner must leave one of its candidates set."""
import numpy as np
import pytest

from conftest import device_buffers, flush_waves, golden_names, load_golden, load_package
import oracle

load_package()

CONFIGS = [(8, 0), (8, 1), (16, 1), (16, 2), (16, 4), (32, 0)]


@pytest.fixture(scope="module")
def ctx():
    from rive_runtime_gb300 import rive_cuda
    c = rive_cuda.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def oracle_images():
    return {n: oracle.render(load_golden(n)[0]) for n in golden_names()}


def _parity(got, want):
    d = np.abs(got.astype(np.int16) - want.astype(np.int16)).max(axis=2)
    return float((d <= 2).mean()), int(d.max())


@pytest.mark.gpu
@pytest.mark.parametrize("config", CONFIGS, ids=lambda c: f"tile{c[0]}_ctas{c[1]}")
def test_every_config_matches_oracle(ctx, oracle_images, config):
    ctx.set_raster_config(*config)
    try:
        assert ctx.raster_config() == (config[0], config[1] if config[0] != 32 else 0)
        for name in golden_names():
            cap = load_golden(name)[0]
            got = ctx.render(cap)
            frac, worst = _parity(got, oracle_images[name])
            assert frac >= 0.999 and worst <= 8, (config, name, frac, worst)
            st = ctx.stats()
            t = config[0]
            # The target's tiles, plus the feather atlas's when the (last)
            # flush renders one.
            d = cap.flushes[-1].desc
            want = ((cap.width + t - 1) // t) * ((cap.height + t - 1) // t)
            if cap.flushes[-1].has_atlas:
                want += (((d["atlas_content_width"] + t - 1) // t) *
                         ((d["atlas_content_height"] + t - 1) // t))
            assert st["tiles"] == want
    finally:
        ctx.set_raster_config(16, 0)


@pytest.mark.gpu
def test_rejects_unknown_tile_size(ctx):
    from rive_runtime_gb300 import rive_cuda
    with pytest.raises(rive_cuda.RiveCudaError):
        ctx.set_raster_config(12, 0)
    with pytest.raises(rive_cuda.RiveCudaError):
        ctx.set_raster_config(16, -1)
    assert ctx.raster_config() == (16, 0)


@pytest.mark.gpu
@pytest.mark.parametrize("tile", [8, 32])
def test_batch_and_graph_at_other_tile_sizes_match_oracle(ctx, oracle_images, tile):
    import torch
    names = golden_names()
    caps = [load_golden(n)[0] for n in names]
    pairs = [device_buffers(c) for c in caps]
    # A stream of its own (graphs launched on a NULL stream run on theirs).
    stream = torch.cuda.Stream().cuda_stream
    ctx.set_raster_config(tile, 0)
    try:
        for mode in ("batch", "graph"):
            targets = [torch.zeros((c.height, c.width, 4), dtype=torch.uint8, device="cuda")
                       for c in caps]
            torch.cuda.synchronize()
            for items in flush_waves(caps, [p[0] for p in pairs], targets):
                if mode == "batch":
                    ctx.flush_batch(items, stream)
                    ctx.sync(stream)
                else:
                    g = ctx.graph(items)
                    g.launch(stream)
                    g.check(stream)
                    g.close()
            torch.cuda.synchronize()
            for name, t in zip(names, targets):
                frac, worst = _parity(t.cpu().numpy(), oracle_images[name])
                assert frac >= 0.999 and worst <= 8, (tile, mode, name, frac, worst)
    finally:
        ctx.set_raster_config(16, 0)


@pytest.mark.gpu
def test_autotune_leaves_a_candidate_set(ctx):
    import torch
    from rive_runtime_gb300 import autotune
    cap = load_golden("full_small_s7")[0]
    bufs, keep = device_buffers(cap)
    target = torch.zeros((cap.height, cap.width, 4), dtype=torch.uint8, device="cuda")
    stream = torch.cuda.Stream()

    def run(s):
        for f in cap.flushes:
            ctx.flush_device(f, bufs, target.data_ptr(), s.cuda_stream)

    try:
        best, trials = autotune.autotune(ctx, run, stream=stream, warmup=1, iters=2)
        assert len(trials) == len(autotune.CANDIDATES)
        assert {(t.tile_size, t.ctas_per_sm) for t in trials} >= {
            (t, c) for t in (8, 16) for c in (1, 2, 4)}
        assert all(t.ms > 0 for t in trials)
        assert ctx.raster_config() == (best.tile_size, best.ctas_per_sm)
        assert ctx.winding_tiles() == best.winding
        assert ctx.raster_queue() == best.queue
        assert best.ms == min(t.ms for t in trials)
    finally:
        ctx.set_raster_config(16, 0)
        ctx.set_winding_tiles(False)
        ctx.set_raster_queue(False)


@pytest.mark.gpu
@pytest.mark.parametrize("ctas", [0, 2])
def test_work_queue_raster_matches_the_grid_bit_for_bit(ctx, ctas):
    """The persistent work-queue raster (heaviest tiles first) renders every
    tile as the one-CTA-per-tile grid does: identical images on every golden,
    one by one, in batches and in graphs."""
    import torch
    names = golden_names()
    caps = [load_golden(n)[0] for n in names]
    ctx.set_raster_config(16, ctas)
    try:
        want = {}
        for queue in (False, True):
            ctx.set_raster_queue(queue)
            assert ctx.raster_queue() == queue
            want[queue] = [ctx.render(c) for c in caps]
        for n, a, b in zip(names, want[False], want[True]):
            assert np.array_equal(a, b), n
        pairs = [device_buffers(c) for c in caps]
        stream = torch.cuda.Stream().cuda_stream
        for mode in ("batch", "graph"):
            targets = [torch.zeros((c.height, c.width, 4), dtype=torch.uint8, device="cuda")
                       for c in caps]
            torch.cuda.synchronize()
            for items in flush_waves(caps, [p[0] for p in pairs], targets):
                if mode == "batch":
                    ctx.flush_batch(items, stream)
                    ctx.sync(stream)
                else:
                    g = ctx.graph(items)
                    g.launch(stream)
                    g.check(stream)
                    g.close()
            torch.cuda.synchronize()
            for n, t, w in zip(names, targets, want[False]):
                assert np.array_equal(t.cpu().numpy(), w), (mode, n)
    finally:
        ctx.set_raster_queue(False)
        ctx.set_raster_config(16, 0)
