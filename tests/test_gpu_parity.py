"""GPU parity: the sm_103a kernels, called through the C ABI, against the
oracle on the golden flush captures of the reference front end.

Tolerances:
  * tessellation: contour IDs and flags bit-exact on every vertex; x, y within
    1e-3 px and theta within 1e-3 rad on >= 99.9% of vertices (the fp32
    algorithm with CUDA's and libm's transcendental functions);
  * gradient ramps: every texel within 1/255 per channel;
  * images: within 2/255 per channel on >= 99.9% of pixels and within 8/255
    everywhere.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden, load_package
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


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_names())
def test_image_matches_oracle(ctx, name):
    cap, _ = load_golden(name)
    got = ctx.render(cap)
    want = oracle.render(cap)
    frac, worst = image_parity(got, want)
    assert frac >= 0.999 and worst <= 8, (name, frac, worst)


@pytest.mark.gpu
@pytest.mark.parametrize("name", golden_names())
def test_tessellation_matches_oracle(ctx, name):
    cap, _ = load_golden(name)
    assert len(cap.flushes) == 1
    ctx.render(cap, read=False)
    h = cap.flushes[0].desc["tess_data_height"]
    got = ctx.read_tess(h)
    want = oracle.tessellate(cap)
    used = want[:, 3] != 0
    assert np.array_equal(got[used, 3], want[used, 3]), name
    gxy = got[used, :2].view(np.float32)
    wxy = want[used, :2].view(np.float32)
    dxy = np.abs(gxy - wxy).max(axis=1)
    # Padding vertices (contour ID 0, all-zero control points) have no
    # defined angle: normalize() of a zero vector, which the GLSL leaves to
    # the implementation's NaN handling. They are never drawn.
    real = (want[used, 3] & 0xFFFF) != 0
    gth = got[used, 2].view(np.float32)[real]
    wth = want[used, 2].view(np.float32)[real]
    assert not np.isnan(wth).any() and not np.isnan(gth).any(), name
    dth = np.abs(gth - wth)
    dth = np.minimum(dth, np.abs(dth - 2 * np.pi))
    assert (dxy <= 1e-3).mean() >= 0.999, (name, float(dxy.max()))
    assert (dth <= 1e-3).mean() >= 0.999, (name, float(dth.max()))


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in golden_names()])
def test_gradient_ramps_match_oracle(ctx, name):
    cap, _ = load_golden(name)
    h = cap.flushes[0].desc["grad_data_height"]
    if cap.flushes[0].desc["grad_span_count"] == 0:
        pytest.skip("no gradients in this scene")
    ctx.render(cap, read=False)
    got = ctx.read_grad(h)
    want = oracle.color_ramps(cap)
    d = np.abs(got.astype(np.int16) - want.astype(np.int16))
    assert d.max() <= 1, (name, int(d.max()))


@pytest.mark.gpu
@pytest.mark.parametrize("draw_type", [4, 5, 6])  # featherAtlasBlit, imageRect, imageMesh
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
