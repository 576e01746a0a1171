"""The batched form (rive_cuda_flush_batch): independent flushes of different
canvases and path counts rendered by one sequence of launches must give every
target exactly the image the one-flush-at-a-time path gives it. Frames of
several logical flushes run as waves: wave i batches logical flush i of every
frame, so a frame's later flushes load what its earlier ones wrote."""
import numpy as np
import pytest

from conftest import (device_buffers, flush_waves, golden_names, load_golden, load_package,
                      render_one_by_one)

load_package()


@pytest.fixture(scope="module")
def ctx():
    from rive_runtime_gb300 import rive_cuda
    c = rive_cuda.Context(0)
    yield c
    c.close()


@pytest.mark.gpu
def test_batch_of_all_goldens_matches_single_flushes(ctx):
    import torch
    names = golden_names()
    caps = [load_golden(n)[0] for n in names]
    assert any(len(c.flushes) > 1 for c in caps), "a multi-flush golden is expected"
    pairs = [device_buffers(c) for c in caps]
    bufs = [p[0] for p in pairs]
    stream = torch.cuda.current_stream().cuda_stream
    want = render_one_by_one(ctx, caps, bufs, stream)
    targets = [torch.zeros((c.height, c.width, 4), dtype=torch.uint8, device="cuda") for c in caps]
    waves = flush_waves(caps, bufs, targets)
    for wave in waves:
        ctx.flush_batch(wave, stream)
    ctx.sync(stream)
    torch.cuda.synchronize()
    for name, t, w in zip(names, targets, want):
        assert np.array_equal(t.cpu().numpy(), w), name
    st = ctx.stats()
    last = [c for c in caps if len(c.flushes) == len(waves)]
    assert st["tiles"] == sum(((c.width + 15) // 16) * ((c.height + 15) // 16) for c in last)


@pytest.mark.gpu
def test_batch_repeats_and_reorders_consistently(ctx):
    """The same scene twice, in different positions of one batch, with another
    scene between: all copies identical to the single-flush image."""
    import torch
    a = load_golden("full_small_s7")[0]
    b = load_golden("strokes_s3")[0]
    (ba, ka), (bb, kb) = device_buffers(a), device_buffers(b)
    stream = torch.cuda.current_stream().cuda_stream
    want_a, want_b = render_one_by_one(ctx, [a, b], [ba, bb], stream)
    ts = [torch.zeros((c.height, c.width, 4), dtype=torch.uint8, device="cuda") for c in (a, b, a)]
    ctx.flush_batch([(a.flushes[0], ba, ts[0].data_ptr()), (b.flushes[0], bb, ts[1].data_ptr()),
                     (a.flushes[0], ba, ts[2].data_ptr())], stream)
    ctx.sync(stream)
    torch.cuda.synchronize()
    assert np.array_equal(ts[0].cpu().numpy(), want_a)
    assert np.array_equal(ts[1].cpu().numpy(), want_b)
    assert np.array_equal(ts[2].cpu().numpy(), want_a)


@pytest.mark.gpu
def test_batch_refuses_a_shared_target(ctx):
    import torch
    from rive_runtime_gb300 import rive_cuda
    a = load_golden("strokes_s3")[0]
    ba, ka = device_buffers(a)
    t = torch.zeros((a.height, a.width, 4), dtype=torch.uint8, device="cuda")
    with pytest.raises(rive_cuda.RiveCudaError, match="share a render target"):
        ctx.flush_batch([(a.flushes[0], ba, t.data_ptr()), (a.flushes[0], ba, t.data_ptr())])
    ctx.flush_batch([])  # an empty batch is a no-op


@pytest.mark.gpu
def test_graph_replays_match_single_flushes(ctx):
    """Each wave captured as a CUDA graph: every replay of the waves, in
    order, gives every target the one-by-one image, and the device status
    stays clean."""
    import torch
    names = golden_names()
    caps = [load_golden(n)[0] for n in names]
    pairs = [device_buffers(c) for c in caps]
    bufs = [p[0] for p in pairs]
    stream = torch.cuda.current_stream().cuda_stream
    want = render_one_by_one(ctx, caps, bufs, stream)
    targets = [torch.zeros((c.height, c.width, 4), dtype=torch.uint8, device="cuda") for c in caps]
    graphs = [ctx.graph(wave) for wave in flush_waves(caps, bufs, targets)]
    # One stream orders the waves (a NULL stream would run each graph on its
    # own stream).
    order = torch.cuda.Stream().cuda_stream
    try:
        for _ in range(2):
            for t in targets:
                t.zero_()
            torch.cuda.synchronize()
            for g in graphs:
                g.launch(order)
            for g in graphs:
                g.check(order)
            torch.cuda.synchronize()
            for name, t, w in zip(names, targets, want):
                assert np.array_equal(t.cpu().numpy(), w), name
        assert all(g.stats()["bin_entries"] > 0 for g in graphs)
    finally:
        for g in graphs:
            g.close()


@pytest.mark.gpu
def test_graph_reports_a_bin_capacity_overflow(ctx):
    """Too small a capacity drops entries on the device and is reported by
    the check (no fault, no out-of-range write); the context stays usable."""
    import torch
    from rive_runtime_gb300 import rive_cuda
    a = load_golden("strokes_s3")[0]
    ba, ka = device_buffers(a)
    t = torch.zeros((a.height, a.width, 4), dtype=torch.uint8, device="cuda")
    g = ctx.graph([(a.flushes[0], ba, t.data_ptr())], bin_capacity=64)
    try:
        g.launch()
        with pytest.raises(rive_cuda.RiveCudaError, match="capacity"):
            g.check()
        g.check()  # the status was cleared
    finally:
        g.close()
    stream = torch.cuda.current_stream().cuda_stream
    (want,) = render_one_by_one(ctx, [a], [ba], stream)
    assert want.any()
