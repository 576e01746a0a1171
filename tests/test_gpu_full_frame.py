"""The benchmarked frame itself, pixel-checked: the full-feature scene at its
stated size (2048x2048, 5,000 paths, seed 2), which the front end splits
into 4 logical flushes, three of them loading the target the earlier ones
wrote (render_context.cpp:509-586 splits, :1218-1222 loads).

  * one frame through rive_cuda_flush against the oracle, at the image
    tolerance (2/255 on >= 99.9% of pixels, 8/255 everywhere);
  * the same frame, beside the two-flush golden, in batches and in CUDA
    graphs (one per wave of logical flushes), bit-identical to flushing one
    logical flush at a time.
"""
import numpy as np
import pytest

from conftest import (device_buffers, flush_waves, load_golden, load_package,
                      render_one_by_one)
import oracle

load_package()


@pytest.fixture(scope="module")
def frame():
    from rive_runtime_gb300 import scene
    from inputgen import planner
    cap = planner.plan(scene.full_feature(seed=2).to_bytes())
    assert (cap.width, cap.height) == (2048, 2048)
    assert len(cap.flushes) == 4
    assert sum(f.desc["color_load_action"] != 0 for f in cap.flushes) == 3
    return cap


@pytest.fixture(scope="module")
def ctx():
    from rive_runtime_gb300 import rive_cuda
    c = rive_cuda.Context(0)
    yield c
    c.close()


@pytest.mark.gpu
def test_full_feature_frame_matches_oracle(ctx, frame):
    got = ctx.render(frame)
    want = oracle.render(frame)
    d = np.abs(got.astype(np.int16) - want.astype(np.int16)).max(axis=2)
    frac, worst = float((d <= 2).mean()), int(d.max())
    print(f"full-feature 2048x2048: {frac:.6f} of pixels within 2/255, worst {worst}/255")
    assert frac >= 0.999 and worst <= 8, (frac, worst)


@pytest.mark.gpu
def test_full_feature_frame_in_batches_and_graphs(ctx, frame):
    import torch
    caps = [frame, load_golden("multiflush_s41")[0]]
    pairs = [device_buffers(c) for c in caps]
    bufs = [p[0] for p in pairs]
    stream = torch.cuda.current_stream().cuda_stream
    want = render_one_by_one(ctx, caps, bufs, stream)
    for mode in ("batch", "graph"):
        targets = [torch.zeros((c.height, c.width, 4), dtype=torch.uint8, device="cuda")
                   for c in caps]
        waves = flush_waves(caps, bufs, targets)
        assert len(waves) == 4
        if mode == "batch":
            for items in waves:
                ctx.flush_batch(items, stream)
            ctx.sync(stream)
        else:
            graphs = [ctx.graph(items) for items in waves]
            # One stream orders the waves (a NULL stream would run each graph
            # on its own stream).
            order = torch.cuda.Stream().cuda_stream
            try:
                for g in graphs:
                    g.launch(order)
                for g in graphs:
                    g.check(order)
            finally:
                for g in graphs:
                    g.close()
        torch.cuda.synchronize()
        for c, t, w in zip(caps, targets, want):
            assert np.array_equal(t.cpu().numpy(), w), (mode, c.width, c.height)
