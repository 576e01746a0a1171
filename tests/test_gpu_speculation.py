"""Speculative bins (rive_cuda_set_bin_speculation): a flush on the context's
own stream enqueues its back half with bins sized from the largest bin-entry
total seen, without waiting for the scan; the total is checked at the next
call and the back half runs again with exact bins when it did not fit.

The images must be bit-identical to exactly sized bins: on frames that fit,
and on a frame far larger than anything the context saw before (every tile's
range emptied, the back half re-run, the read-back enqueued behind it
repeated)."""
import numpy as np
import pytest
import torch

from conftest import load_golden, load_package

load_package()

SMALL = "plain_small_s1"
LARGE = ["full_odd_s11", "multiflush_s41", "silver_hunter_x_f0", "image_meshes_s43"]


def _render(ctx, cap):
    """Uploads and flushes `cap` on the context's stream, then reads the
    target back asynchronously into pinned host memory (the read-back is
    enqueued behind the last flush) and syncs."""
    t = ctx.render_target(cap.width, cap.height)
    ctx.upload_frame(cap)
    for f in cap.flushes:
        ctx.flush(f, t)
    out = torch.empty((cap.height, cap.width, 4), dtype=torch.uint8).pin_memory()
    ctx.read_target_async(t, out.data_ptr())
    ctx.sync()
    return out.numpy().copy()


@pytest.fixture(scope="module")
def exact():
    from rive_runtime_gb300 import rive_cuda
    c = rive_cuda.Context(0)
    c.set_bin_speculation(False)
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", LARGE)
def test_speculative_bins_match_exact_bins(exact, name):
    from rive_runtime_gb300 import rive_cuda
    small, _ = load_golden(SMALL)
    cap, _ = load_golden(name)
    want = _render(exact, cap)
    ctx = rive_cuda.Context(0)
    try:
        # A small frame first: the first flush sizes exactly and sets the
        # high-water mark far below this frame's total, so its first
        # speculative flush falls short and runs again.
        _render(ctx, small)
        got = _render(ctx, cap)
        assert np.array_equal(got, want), name
        # Now the mark covers it: the same frame fits and still matches.
        got = _render(ctx, cap)
        assert np.array_equal(got, want), name
        # The stats settle to the exact total of the last flush.
        assert ctx.stats()["bin_entries"] == exact.stats()["bin_entries"] > 0
    finally:
        ctx.close()


@pytest.mark.gpu
def test_speculation_is_on_by_default_and_switchable():
    import ctypes
    from rive_runtime_gb300 import rive_cuda
    ctx = rive_cuda.Context(0)
    try:
        v = ctypes.c_int(-1)
        assert ctx.lib.rive_cuda_get_bin_speculation(ctx.h, ctypes.byref(v)) == 0
        assert v.value == 1
        ctx.set_bin_speculation(False)
        assert ctx.lib.rive_cuda_get_bin_speculation(ctx.h, ctypes.byref(v)) == 0
        assert v.value == 0
    finally:
        ctx.close()


@pytest.mark.gpu
def test_flushes_on_two_streams_run_in_issue_order(exact):
    """A speculative flush on the context's stream, then at once a flush of
    another frame on a caller's stream into caller-owned memory: they share
    the context's intermediates, so the second waits for the first; both
    images equal exactly sized, one-stream renders."""
    from conftest import device_buffers
    from rive_runtime_gb300 import rive_cuda
    a, _ = load_golden("full_odd_s11")
    b, _ = load_golden("silver_hunter_x_f0")
    want_a = _render(exact, a)
    want_b = _render(exact, b)
    ctx = rive_cuda.Context(0)
    try:
        _render(ctx, a)  # a total seen: the next flushes speculate
        bufs, keep = device_buffers(b)
        side = torch.cuda.Stream()
        out_b = torch.zeros((b.height, b.width, 4), dtype=torch.uint8, device="cuda")
        t = ctx.render_target(a.width, a.height)
        ctx.upload_frame(a)
        for f in a.flushes:
            ctx.flush(f, t)
        for f in b.flushes:
            ctx.flush_device(f, bufs, out_b.data_ptr(), side.cuda_stream)
        got_a = ctx.read_target(t, a.width, a.height)
        ctx.sync(side.cuda_stream)
        assert np.array_equal(got_a, want_a)
        assert np.array_equal(out_b.cpu().numpy(), want_b)
    finally:
        ctx.close()
