"""The batched form (rive_cuda_flush_batch): independent flushes of different
canvases and path counts rendered by one sequence of launches must give every
target exactly the image the one-flush-at-a-time path gives it."""
import numpy as np
import pytest

from conftest import golden_names, load_golden, load_package

load_package()


def _device_buffers(cap):
    import torch
    from rive_runtime_gb300 import rive_cuda
    from rive_runtime_gb300.capture import BUFFER_NAMES
    bufs = rive_cuda.DeviceBuffers()
    keep = []
    for name in BUFFER_NAMES:
        b = cap.buffers.get(name, b"")
        t = torch.from_numpy(np.frombuffer(b, np.uint8).copy()).cuda() if b else None
        keep.append(t)
        setattr(bufs, name, t.data_ptr() if t is not None else None)
    return bufs, keep


@pytest.fixture(scope="module")
def ctx():
    from rive_runtime_gb300 import rive_cuda
    c = rive_cuda.Context(0)
    yield c
    c.close()


def _one_by_one(ctx, caps, bufs, stream):
    import torch
    out = []
    for cap, b in zip(caps, bufs):
        t = torch.zeros((cap.height, cap.width, 4), dtype=torch.uint8, device="cuda")
        for f in cap.flushes:
            ctx.flush_device(f, b, t.data_ptr(), stream)
        out.append(t)
    ctx.sync(stream)
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in out]


@pytest.mark.gpu
def test_batch_of_all_goldens_matches_single_flushes(ctx):
    import torch
    caps = [load_golden(n)[0] for n in golden_names()]
    assert all(len(c.flushes) == 1 for c in caps)
    pairs = [_device_buffers(c) for c in caps]
    bufs = [p[0] for p in pairs]
    stream = torch.cuda.current_stream().cuda_stream
    want = _one_by_one(ctx, caps, bufs, stream)
    targets = [torch.zeros((c.height, c.width, 4), dtype=torch.uint8, device="cuda") for c in caps]
    ctx.flush_batch([(c.flushes[0], b, t.data_ptr()) for c, b, t in zip(caps, bufs, targets)],
                    stream)
    ctx.sync(stream)
    torch.cuda.synchronize()
    for name, t, w in zip(golden_names(), targets, want):
        assert np.array_equal(t.cpu().numpy(), w), name
    st = ctx.stats()
    assert st["tiles"] == sum(((c.width + 15) // 16) * ((c.height + 15) // 16) for c in caps)


@pytest.mark.gpu
def test_batch_repeats_and_reorders_consistently(ctx):
    """The same scene twice, in different positions of one batch, with another
    scene between: all copies identical to the single-flush image."""
    import torch
    a = load_golden("full_small_s7")[0]
    b = load_golden("strokes_s3")[0]
    (ba, ka), (bb, kb) = _device_buffers(a), _device_buffers(b)
    stream = torch.cuda.current_stream().cuda_stream
    want_a, want_b = _one_by_one(ctx, [a, b], [ba, bb], stream)
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
    ba, ka = _device_buffers(a)
    t = torch.zeros((a.height, a.width, 4), dtype=torch.uint8, device="cuda")
    with pytest.raises(rive_cuda.RiveCudaError, match="share a render target"):
        ctx.flush_batch([(a.flushes[0], ba, t.data_ptr()), (a.flushes[0], ba, t.data_ptr())])
    ctx.flush_batch([])  # an empty batch is a no-op


@pytest.mark.gpu
def test_graph_replays_match_single_flushes(ctx):
    """A batch captured as a CUDA graph: every launch gives every target the
    one-by-one image, and the device status stays clean."""
    import torch
    caps = [load_golden(n)[0] for n in golden_names()]
    pairs = [_device_buffers(c) for c in caps]
    bufs = [p[0] for p in pairs]
    stream = torch.cuda.current_stream().cuda_stream
    want = _one_by_one(ctx, caps, bufs, stream)
    targets = [torch.zeros((c.height, c.width, 4), dtype=torch.uint8, device="cuda") for c in caps]
    g = ctx.graph([(c.flushes[0], b, t.data_ptr()) for c, b, t in zip(caps, bufs, targets)])
    try:
        for _ in range(2):
            for t in targets:
                t.zero_()
            torch.cuda.synchronize()
            g.launch()
            g.check()
            torch.cuda.synchronize()
            for name, t, w in zip(golden_names(), targets, want):
                assert np.array_equal(t.cpu().numpy(), w), name
        assert g.stats()["bin_entries"] > 0
    finally:
        g.close()


@pytest.mark.gpu
def test_graph_reports_a_bin_capacity_overflow(ctx):
    """Too small a capacity drops entries on the device and is reported by
    the check (no fault, no out-of-range write); the context stays usable."""
    import torch
    from rive_runtime_gb300 import rive_cuda
    a = load_golden("strokes_s3")[0]
    ba, ka = _device_buffers(a)
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
    (want,) = _one_by_one(ctx, [a], [ba], stream)
    assert want.any()
