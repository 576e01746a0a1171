"""Image paints (RiveRenderer::drawImage in rasterOrdering: a rectangle path
with an image paint, rive_renderer.cpp:383-446; ENABLE_MODULATED_IMAGE,
draw_path.vert:343-361, 478-493).

CPU: the capture carries the textures the front end created
(RenderContextImpl::makeImageTexture) and each draw batch's texture and
sampler. GPU: the device mip chains equal the oracle's bit for bit; the
images of every golden, image frames included, are checked against the
oracle by test_gpu_parity.py (in batches and graphs by test_gpu_batch.py, at
every raster configuration by test_gpu_raster_config.py)."""
import ctypes

import numpy as np
import pytest

from conftest import GOLDEN, load_golden
import oracle

IMAGE_GOLDENS = ["images_s41"]


@pytest.mark.parametrize("name", IMAGE_GOLDENS)
def test_image_goldens_carry_textures_and_batch_images(name):
    from rive_runtime_gb300 import capture
    cap, _ = load_golden(name)
    assert cap.textures
    for t in cap.textures:
        assert len(t.rgba) == t.width * t.height * 4
        # The reference asks for the full chain: msb(width | height) levels
        # (render_context.cpp:251).
        assert t.mip_levels == (t.width | t.height).bit_length()
    f = cap.flushes[0]
    assert f.has_images and len(f.images) == len(f.batches)
    used = f.images[f.images[:, 0] != 0xFFFFFFFF]
    assert (used[:, 0] < len(cap.textures)).all() and (used[:, 1] < 18).all()
    # Every ImageSampler the scene draws with appears in some batch.
    assert len(set(used[:, 1].tolist())) > 4
    # Batches with an image carry ENABLE_MODULATED_IMAGE.
    assert (f.batches[f.images[:, 0] != 0xFFFFFFFF, 3] & (1 << 8)).all()
    with open(f"{GOLDEN}/{name}.cap", "rb") as fh:
        raw = fh.read()
    assert capture.serialize(capture.parse(raw)) == raw


def _oracle_mips(texture):
    """The oracle's mip levels of a capture texture, as (h, w, 4) arrays."""
    (ot, _, _), = oracle._textures([texture])
    out = []
    for level in range(texture.mip_levels):
        w, h = max(texture.width >> level, 1), max(texture.height >> level, 1)
        addr = ot.mips + ot.off[level] * 4
        out.append(np.ctypeslib.as_array((ctypes.c_uint8 * (w * h * 4)).from_address(addr))
                   .reshape(h, w, 4).copy())
    return out


def test_oracle_mip_chain_is_the_rounded_two_by_two_mean():
    cap, _ = load_golden("images_s41")
    t = next(t for t in cap.textures if t.width % 2 or t.height % 2)  # an odd size
    mips = _oracle_mips(t)
    for level in range(1, t.mip_levels):
        src, dst = mips[level - 1].astype(np.uint32), mips[level]
        sh, sw = src.shape[:2]
        for y in range(dst.shape[0]):
            for x in range(dst.shape[1]):
                xs = [min(2 * x, sw - 1), min(2 * x + 1, sw - 1)]
                ys = [min(2 * y, sh - 1), min(2 * y + 1, sh - 1)]
                want = (src[ys[0], xs[0]] + src[ys[0], xs[1]] + src[ys[1], xs[0]]
                        + src[ys[1], xs[1]] + 2) >> 2
                assert np.array_equal(dst[y, x], want.astype(np.uint8)), (level, x, y)


@pytest.fixture(scope="module")
def ctx():
    from rive_runtime_gb300 import rive_cuda
    c = rive_cuda.Context(0)
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", IMAGE_GOLDENS)
def test_device_mip_chains_equal_the_oracle(ctx, name):
    cap, _ = load_golden(name)
    handles = ctx.textures_for(cap.flushes[0])
    for t, h in zip(cap.textures, handles):
        want = _oracle_mips(t)
        for level in range(t.mip_levels):
            w, hh = max(t.width >> level, 1), max(t.height >> level, 1)
            got = ctx.read_texture(h, level, w, hh)
            assert np.array_equal(got, want[level]), (name, t.width, t.height, level)
