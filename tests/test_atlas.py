"""The feather atlas (render_context.cpp:676-744, 2255-2345, 3515-3534;
render_atlas.glsl; draw_mesh.frag with FEATHER_ATLAS_BLIT).

CPU: the captures that carry atlas batches, and the oracle's atlas pass pinned
against the reference's own direct feathers: the same scene recorded with
PlatformFeatures::alwaysFeatherToAtlas renders the image its direct feathers
render. GPU: the kernel's atlas texels against the oracle's, and the same twin
comparison on the device (every golden's image, atlas ones included, is also
checked against the oracle by test_gpu_parity.py, in batches and graphs by
test_gpu_batch.py and at every raster configuration by
test_gpu_raster_config.py)."""
import numpy as np
import pytest

from conftest import GOLDEN, device_buffers, load_golden
import oracle

ATLAS_GOLDENS = ["feather_atlas_s35", "feathered_atlas_s33", "silver_data_viz_f6",
                 "silver_bankcard_f10", "silver_rewards_atlas_f10"]


def image_parity(a, b):
    d = np.abs(a.astype(np.int16) - b.astype(np.int16)).max(axis=-1)
    return float((d <= 2).mean()), int(d.max())


@pytest.mark.parametrize("name", ATLAS_GOLDENS)
def test_atlas_goldens_carry_atlas_batches(name):
    from rive_runtime_gb300 import capture
    cap, _ = load_golden(name)
    with_atlas = [f for f in cap.flushes if f.has_atlas]
    assert with_atlas
    for f in with_atlas:
        d = f.desc
        n = d["atlas_fill_batch_count"] + d["atlas_stroke_batch_count"]
        assert len(f.atlas) == n > 0
        assert 0 < d["atlas_content_width"] <= d["atlas_texture_width"]
        assert 0 < d["atlas_content_height"] <= d["atlas_texture_height"]
        left, top = f.atlas[:, 0] & 0xffff, f.atlas[:, 0] >> 16
        right, bottom = f.atlas[:, 1] & 0xffff, f.atlas[:, 1] >> 16
        assert (left <= right).all() and (top <= bottom).all()
        assert (right <= d["atlas_content_width"]).all()
        assert (bottom <= d["atlas_content_height"]).all()
        # Every atlas draw is blitted by a featherAtlasBlit batch (draw type
        # 4): one rectangle, six triangle vertices, per path.
        blits = f.batches[f.batches[:, 0] == 4]
        assert len(blits) and (blits[:, 1] % 6 == 0).all()
    # RCP2 captures round-trip through the Python writer byte for byte.
    with open(f"{GOLDEN}/{name}.cap", "rb") as fh:
        raw = fh.read()
    assert capture.serialize(capture.parse(raw)) == raw


def test_atlas_twin_renders_like_direct_feathers():
    """feathered_atlas_s33 is feathered_s33 with every feather through the
    atlas: the reference front end blits coverage rendered offscreen instead
    of feathering in the main pass. The oracle's two images agree within the
    image tolerance, so its atlas pass and blits restate the same coverage as
    its (reference-pinned) direct feathers."""
    direct = oracle.render(load_golden("feathered_s33")[0])
    atlas = oracle.render(load_golden("feathered_atlas_s33")[0])
    frac, worst = image_parity(atlas, direct)
    assert frac >= 0.999 and worst <= 8, (frac, worst)


def test_oracle_atlas_is_deterministic_across_threads():
    cap, _ = load_golden("feather_atlas_s35")
    a = oracle.atlas(cap, 0, threads=1)
    b = oracle.atlas(cap, 0, threads=4)
    assert np.array_equal(a, b)
    assert a.max() > 0.5  # something was drawn


@pytest.fixture(scope="module")
def ctx():
    from rive_runtime_gb300 import rive_cuda
    c = rive_cuda.Context(0)
    yield c
    c.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ATLAS_GOLDENS)
def test_atlas_texels_match_oracle(ctx, name):
    """The atlas pass alone: every texel the kernel stores against the
    oracle's, flush by flush. Both round each blend to fp16; they differ only
    where the kernel's plane evaluation of a coverage lands an fp16 rounding
    step away from the oracle's barycentric one, or where a texel centre lies
    on a triangle edge (the kernel tests edges in tile-local floats, the
    oracle in exact integers)."""
    cap, _ = load_golden(name)
    t = ctx.render_target(cap.width, cap.height)
    ctx.upload_frame(cap)
    worst = 0.0
    for i, f in enumerate(cap.flushes):
        ctx.flush(f, t)
        ctx.sync()
        if not f.has_atlas:
            continue
        w, h = f.desc["atlas_content_width"], f.desc["atlas_content_height"]
        got = ctx.read_atlas(w, h)
        want = oracle.atlas(cap, i)
        d = np.abs(got - want)
        assert (d <= 1 / 256).mean() >= 0.999, (name, i, float((d <= 1 / 256).mean()))
        assert d.max() <= 1 / 8, (name, i, float(d.max()))
        worst = max(worst, float(d.max()))
    print(f"{name}: worst atlas texel difference {worst:.4g}")


@pytest.mark.gpu
def test_atlas_twin_matches_direct_feathers_on_the_gpu(ctx):
    direct = ctx.render(load_golden("feathered_s33")[0])
    atlas = ctx.render(load_golden("feathered_atlas_s33")[0])
    frac, worst = image_parity(atlas, direct)
    assert frac >= 0.999 and worst <= 8, (frac, worst)


@pytest.mark.gpu
def test_atlas_frames_render_in_one_batch_like_one_by_one(ctx):
    """The atlas scenes of several flushes share one batch: each target equals
    its own flush rendered alone."""
    import torch
    from conftest import render_one_by_one
    caps = [load_golden(n)[0] for n in ATLAS_GOLDENS]
    pairs = [device_buffers(c) for c in caps]
    bufs = [p[0] for p in pairs]
    stream = torch.cuda.Stream()
    alone = render_one_by_one(ctx, caps, bufs, stream.cuda_stream)
    targets = [torch.zeros((c.height, c.width, 4), dtype=torch.uint8, device="cuda") for c in caps]
    n = max(len(c.flushes) for c in caps)
    for wave in range(n):
        items = [(c.flushes[wave], b, t.data_ptr()) for c, b, t in zip(caps, bufs, targets)
                 if wave < len(c.flushes)]
        ctx.flush_batch(items, stream.cuda_stream)
    ctx.sync(stream.cuda_stream)
    torch.cuda.synchronize()
    for name, a, t in zip(ATLAS_GOLDENS, alone, targets):
        assert np.array_equal(a, t.cpu().numpy()), name
