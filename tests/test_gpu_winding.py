"""Interior tiles as winding records (rive_cuda_set_winding_tiles) against
the plain midpoint fan, kernel against kernel: on every golden, on the
full-feature 2048x2048 frame, at every tile size and in batches, the images
must be bit-identical (the winding entry adds the fan's integer coverage sum
once, and integer sums are exact in the fp16 coverage plane whatever their
order), and the winding entries must replace fan entries (fewer bin entries
where fills have interiors)."""
import numpy as np
import pytest

from conftest import (device_buffers, flush_waves, golden_names, load_golden, load_package)

load_package()


@pytest.fixture(scope="module")
def ctx():
    from rive_runtime_gb300 import rive_cuda
    c = rive_cuda.Context(0)
    yield c
    c.close()


def _render(ctx, cap, winding):
    ctx.set_winding_tiles(winding)
    try:
        img = ctx.render(cap)
        return img, ctx.stats()
    finally:
        ctx.set_winding_tiles(False)


@pytest.mark.gpu
def test_winding_tiles_are_off_by_default(ctx):
    assert not ctx.winding_tiles()


@pytest.mark.gpu
@pytest.mark.parametrize("tile", [16, 8, 32])
@pytest.mark.parametrize("name", golden_names())
def test_winding_tiles_match_the_fan_bit_for_bit(ctx, name, tile):
    cap, _ = load_golden(name)
    ctx.set_raster_config(tile, 0)
    try:
        fan, sf = _render(ctx, cap, False)
        wind, sw = _render(ctx, cap, True)
    finally:
        ctx.set_raster_config(16, 0)
    assert sf["winding_entries"] == 0
    assert np.array_equal(wind, fan), (name, tile, int((wind != fan).any(axis=2).sum()))
    if sw["winding_entries"]:
        assert sw["bin_entries"] < sf["bin_entries"], (name, sw, sf)


@pytest.mark.gpu
def test_full_feature_frame_winding_matches_the_fan(ctx):
    from rive_runtime_gb300 import scene
    from inputgen import planner
    cap = planner.plan(scene.full_feature(seed=2).to_bytes())
    fan, sf = _render(ctx, cap, False)
    wind, sw = _render(ctx, cap, True)
    print(f"full-feature last flush: bin entries {sf['bin_entries']} with the fan, "
          f"{sw['bin_entries']} with winding records ({sw['winding_entries']} of them)")
    assert np.array_equal(wind, fan), int((wind != fan).any(axis=2).sum())
    assert sw["bin_entries"] <= sf["bin_entries"]


@pytest.mark.gpu
def test_batched_winding_matches_the_fan(ctx):
    import torch
    names = golden_names()
    caps = [load_golden(n)[0] for n in names]
    pairs = [device_buffers(c) for c in caps]
    bufs = [p[0] for p in pairs]
    stream = torch.cuda.Stream().cuda_stream
    images = {}
    for winding in (False, True):
        ctx.set_winding_tiles(winding)
        targets = [torch.zeros((c.height, c.width, 4), dtype=torch.uint8, device="cuda")
                   for c in caps]
        torch.cuda.synchronize()
        for items in flush_waves(caps, bufs, targets):
            ctx.flush_batch(items, stream)
        ctx.sync(stream)
        torch.cuda.synchronize()
        images[winding] = [t.cpu().numpy() for t in targets]
    ctx.set_winding_tiles(False)
    for name, a, b in zip(names, images[False], images[True]):
        assert np.array_equal(a, b), name


@pytest.mark.gpu
def test_graph_winding_matches_the_fan(ctx):
    import torch
    cap = load_golden("plain_small_s1")[0]
    bufs, keep = device_buffers(cap)
    stream = torch.cuda.Stream().cuda_stream
    out = {}
    for winding in (False, True):
        ctx.set_winding_tiles(winding)
        t = torch.zeros((cap.height, cap.width, 4), dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        g = ctx.graph([(cap.flushes[0], bufs, t.data_ptr())])
        try:
            for _ in range(2):
                g.launch(stream)
                g.check(stream)
        finally:
            g.close()
        out[winding] = t.cpu().numpy()
    ctx.set_winding_tiles(False)
    assert np.array_equal(out[False], out[True])
