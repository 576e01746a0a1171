"""GPU parity: the sm_103a kernels, called through the C ABI, against the
oracle on the golden flush captures of the reference front end.

Tolerances:
  * tessellation: every texel of every logical flush bit-exact against the
    oracle's fp32 tessellator (x, y, theta, contourIDWithFlags; both evaluate
    the same operations with the same elementary functions), and every used
    vertex within 1e-4 px of the FP64 evaluation of its segment parameters,
    or within 1 ulp of its coordinate where fp32 spacing itself exceeds that
    (coordinates beyond 1,024 px; the compensated evaluation keeps it within
    half an ulp);
  * gradient ramps: every texel within 1/255 per channel;
  * images: within 2/255 per channel on >= 99.9% of pixels and within 8/255
    everywhere.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden, load_package, tess_written
import oracle

load_package()


@pytest.fixture(scope="module")
def ctx():
    from rive_runtime_gb300 import rive_cuda
    c = rive_cuda.Context(0)
    yield c
    c.close()


def image_parity(got, want):
    d = np.abs(got.astype(np.int16) - want.astype(np.int16)).max(axis=2)
    return float((d <= 2).mean()), int(d.max())


def flush_by_flush(ctx, cap, after_flush):
    """Uploads the frame and runs its logical flushes one at a time, calling
    after_flush(i) once flush i has finished on the device."""
    t = ctx.render_target(cap.width, cap.height)
    ctx.upload_frame(cap)
    for i, f in enumerate(cap.flushes):
        ctx.flush(f, t)
        ctx.sync()
        after_flush(i)
    return t


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_names())
def test_image_matches_oracle(ctx, name):
    cap, _ = load_golden(name)
    got = ctx.render(cap)
    want = oracle.render(cap)
    frac, worst = image_parity(got, want)
    assert frac >= 0.999 and worst <= 8, (name, frac, worst)


def test_a_golden_splits_into_logical_flushes():
    """The multi-flush golden covers what the bench frame does: later logical
    flushes load the target the earlier ones wrote."""
    cap, _ = load_golden("multiflush_s41")
    assert len(cap.flushes) == 2
    assert cap.flushes[0].desc["color_load_action"] != cap.flushes[1].desc["color_load_action"]


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_names())
def test_tessellation_matches_oracle(ctx, name):
    cap, _ = load_golden(name)
    worst = [0.0]

    if not any(f.desc["tess_span_count"] for f in cap.flushes):
        pytest.skip("no tessellation in this scene")

    def check(i):
        h = cap.flushes[i].desc["tess_data_height"]
        if not cap.flushes[i].desc["tess_span_count"]:
            return
        written = tess_written(cap, i)
        got = ctx.read_tess(h)[written]
        want = oracle.tessellate(cap, i)[written]
        assert np.array_equal(got, want), (name, i, int((got != want).any(axis=1).sum()))
        xy64, flags64 = oracle.tessellate_f64(cap, i)
        xy64, flags64 = xy64[written], flags64[written]
        used = flags64 != 0
        xy = got[used, :2].view(np.float32).astype(np.float64)
        err = np.abs(xy - xy64[used])
        ulp = np.spacing(np.abs(xy64[used]).astype(np.float32)).astype(np.float64)
        assert (err <= np.maximum(1e-4, ulp)).all(), (name, i, float(err.max()))
        worst[0] = max(worst[0], float(err.max()) if err.size else 0.0)

    flush_by_flush(ctx, cap, check)
    print(f"{name}: worst vertex error vs FP64 {worst[0]:.3g} px")


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_names())
def test_gradient_ramps_match_oracle(ctx, name):
    cap, _ = load_golden(name)
    if all(f.desc["grad_span_count"] == 0 for f in cap.flushes):
        pytest.skip("no gradients in this scene")

    def check(i):
        h = cap.flushes[i].desc["grad_data_height"]
        if cap.flushes[i].desc["grad_span_count"] == 0:
            return
        got = ctx.read_grad(h)
        want = oracle.color_ramps(cap, i)
        d = np.abs(got.astype(np.int16) - want.astype(np.int16))
        assert d.max() <= 1, (name, i, int(d.max()))

    flush_by_flush(ctx, cap, check)


@pytest.mark.gpu
@pytest.mark.parametrize("draw_type", [5, 7])  # imageRect (atomic mode), msaaStrokes
def test_flush_rejects_unsupported_draw_type_and_stays_usable(ctx, draw_type):
    from rive_runtime_gb300 import rive_cuda
    cap, _ = load_golden("plain_small_s1")
    f = cap.flushes[0]
    bad = type(f)(dict(f.desc), f.batches.copy())
    bad.batches[:, 0] = draw_type
    t = ctx.render_target(cap.width, cap.height)
    ctx.upload_frame(cap)
    with pytest.raises(rive_cuda.RiveCudaError, match="draw type"):
        ctx.flush(bad, t)
    got = ctx.render(cap)
    frac, worst = image_parity(got, oracle.render(cap))
    assert frac >= 0.999 and worst <= 8


@pytest.mark.gpu
def test_flush_rejects_an_image_mesh_without_buffers(ctx):
    """An imageMesh batch (draw type 6) with no rive_cuda_batch_mesh is
    refused on the host before anything runs."""
    from rive_runtime_gb300 import rive_cuda
    cap, _ = load_golden("plain_small_s1")
    f = cap.flushes[0]
    bad = type(f)(dict(f.desc), f.batches.copy())
    bad.batches[:, 0] = 6
    t = ctx.render_target(cap.width, cap.height)
    ctx.upload_frame(cap)
    with pytest.raises(rive_cuda.RiveCudaError, match="image mesh batch"):
        ctx.flush(bad, t)


@pytest.mark.gpu
def test_repeated_frames_are_identical(ctx):
    cap, _ = load_golden("full_small_s7")
    a = ctx.render(cap)
    b = ctx.render(cap)
    assert np.array_equal(a, b)


@pytest.mark.gpu
def test_async_read_back_equals_sync_read_back(ctx):
    """rive_cuda_render_target_read_async lands the same pixels as the
    synchronous read once the stream is synced, even with the next frame's
    flush already enqueued behind it."""
    import torch
    cap, _ = load_golden("full_small_s7")
    other, _ = load_golden("strokes_s3")  # same 256x256 canvas
    assert (other.width, other.height) == (cap.width, cap.height)
    t = ctx.render_target(cap.width, cap.height)
    want = ctx.render(cap, target=t)
    out = torch.zeros((cap.height, cap.width, 4), dtype=torch.uint8).pin_memory()
    ctx.read_target_async(t, out.data_ptr())
    # A later frame on the same stream overwrites the target after the copy.
    ctx.upload_frame(other)
    for f in other.flushes:
        ctx.flush(f, t)
    ctx.sync()
    assert np.array_equal(out.numpy(), want)
    assert not np.array_equal(ctx.read_target(t, cap.width, cap.height), want)
