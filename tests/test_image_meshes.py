"""Image meshes (RiveRenderer::drawImageMesh, rive_renderer.cpp:448-495;
draw_image_mesh.vert, draw_mesh.frag with DRAW_IMAGE_MESH).

CPU: the capture carries each imageMesh batch's RenderBuffers (vertex
positions, texture coordinates, uint16 indices), its index count and the
ImageDrawInstance records; the oracle's mip-level rule and its per-triangle
blending are pinned on known answers. GPU: the golden's image against the
oracle is checked by test_gpu_parity.py (in batches and graphs by
test_gpu_batch.py, at every raster configuration by
test_gpu_raster_config.py); here, a bad index is reported through the device
status word without touching memory out of bounds."""
import copy
import math

import numpy as np
import pytest

from conftest import GOLDEN, load_golden, load_package
import oracle

load_package()
from rive_runtime_gb300 import capture, scene  # noqa: E402

MESH_GOLDENS = ["image_meshes_s43"]
DRAW_IMAGE_MESH = 6


@pytest.mark.parametrize("name", MESH_GOLDENS)
def test_mesh_goldens_carry_buffers_and_instances(name):
    cap, _ = load_golden(name)
    f = cap.flushes[0]
    assert f.has_meshes and len(f.meshes) == len(f.batches)
    mesh_batches = np.nonzero(f.batches[:, 0] == DRAW_IMAGE_MESH)[0]
    assert len(mesh_batches) > 10
    # One ImageDrawInstance (64 bytes) per mesh batch, each its own instance
    # (image draws never merge, render_context.cpp:3952-3957).
    assert len(cap.buffers["image_draws"]) == 64 * len(mesh_batches)
    assert sorted(f.batches[mesh_batches, 2].tolist()) == list(range(len(mesh_batches)))
    assert (f.batches[mesh_batches, 1] == 1).all()
    for b in mesh_batches:
        vb, ub, ib, n = (int(v) for v in f.meshes[b])
        assert n % 3 == 0 and n > 0
        assert cap.render_buffers[vb].type == 1 and cap.render_buffers[ub].type == 1
        assert cap.render_buffers[ib].type == 0
        nv = len(cap.render_buffers[vb].data) // 8
        assert len(cap.render_buffers[ub].data) // 8 == nv
        idx = np.frombuffer(cap.render_buffers[ib].data, np.uint16)[:n]
        assert (idx < nv).all()
        # Every mesh samples a texture.
        assert f.images[b, 0] != 0xFFFFFFFF
    # Batches that are not meshes name no buffers.
    assert (f.meshes[f.batches[:, 0] != DRAW_IMAGE_MESH, 0] == 0xFFFFFFFF).all()
    with open(f"{GOLDEN}/{name}.cap", "rb") as fh:
        raw = fh.read()
    assert raw[:4] == b"RCP3"
    assert capture.serialize(capture.parse(raw)) == raw


def test_mesh_mip_level_known_answers():
    # lambda = log2(rho) - 1/2 (MIP_MAP_LOD_BIAS, gpu.hpp:52); nearest mip
    # ceil(lambda + 1/2) - 1: level k from rho > 2^k, i.e. rho^2 > 4^k.
    cases = [(0.0, 0), (1.0, 0), (3.99, 0), (4.0, 0), (4.0001, 1), (16.0, 1),
             (16.01, 2), (4.0 ** 5 + 1, 5), (float("inf"), 15), (float("nan"), 0)]
    for rho2, want in cases:
        assert oracle.mesh_mip_level(rho2, -0.5, 16) == want, rho2
    # Clamped to the texture's last level.
    assert oracle.mesh_mip_level(1e12, -0.5, 4) == 3
    assert oracle.mesh_mip_level(1e12, -0.5, 1) == 0
    # A bias of 0: lambda = log2(rho); level k from rho > 2^(k - 1/2).
    assert oracle.mesh_mip_level(1.99, 0.0, 16) == 0
    assert oracle.mesh_mip_level(2.01, 0.0, 16) == 1
    assert oracle.mesh_mip_level(8.01, 0.0, 16) == 2
    # Against the formula itself, away from the half-integer boundaries.
    rng = np.random.default_rng(3)
    for rho in np.exp(rng.uniform(-3, 8, 200)):
        lam = math.log2(rho) - 0.5
        if abs(lam - round(lam - 0.5) - 0.5) < 1e-3:
            continue
        want = 0 if lam <= 0.5 else min(math.ceil(lam + 0.5) - 1, 9)
        assert oracle.mesh_mip_level(float(rho) ** 2, -0.5, 10) == want, rho


def test_oracle_blends_every_covering_triangle():
    cap, _ = load_golden("mesh_overlap")
    img = oracle.render(cap)
    # Outside: white. One triangle: white * 1/2 + red * 1/2. Both (the
    # second faces the other way and is drawn too): that again.
    assert tuple(img[2, 2]) == (255, 255, 255, 255)
    assert tuple(img[10, 10]) == (255, 128, 128, 255)
    assert tuple(img[20, 20]) == (255, 64, 64, 255)
    assert tuple(img[50, 40]) == (255, 255, 255, 255)


@pytest.fixture(scope="module")
def ctx():
    from rive_runtime_gb300 import rive_cuda
    c = rive_cuda.Context(0)
    yield c
    c.close()


@pytest.mark.gpu
def test_gpu_blends_every_covering_triangle(ctx):
    cap, _ = load_golden("mesh_overlap")
    got = ctx.render(cap)
    assert tuple(got[10, 10]) == (255, 128, 128, 255)
    assert tuple(got[20, 20]) == (255, 64, 64, 255)
    assert np.array_equal(got, oracle.render(cap))


@pytest.mark.gpu
@pytest.mark.parametrize("name", MESH_GOLDENS)
def test_bad_mesh_index_sets_the_device_status(ctx, name):
    """An index past the mesh's vertices: the triangle is dropped and the
    device status word reports it (bit 64); the context stays usable."""
    from rive_runtime_gb300.rive_cuda import RiveCudaError
    cap, _ = load_golden(name)
    bad = copy.copy(cap)
    bad.render_buffers = list(cap.render_buffers)
    f = copy.copy(cap.flushes[0])
    b = int(np.nonzero(f.batches[:, 0] == DRAW_IMAGE_MESH)[0][0])
    vb, _, ib, n = (int(v) for v in f.meshes[b])
    nv = len(cap.render_buffers[vb].data) // 8
    idx = np.frombuffer(cap.render_buffers[ib].data, np.uint16).copy()
    idx[1] = nv  # one past the last vertex
    bad.render_buffers[ib] = capture.RenderBuffer(0, idx.tobytes())
    f.render_buffers = bad.render_buffers
    bad.flushes = [f]
    with pytest.raises(RiveCudaError, match="64 mesh index|0x40"):
        ctx.render(bad)
    # The status was cleared: the same context renders the unmodified frame.
    assert ctx.render(cap).shape == (cap.height, cap.width, 4)
