"""rive_cuda_flush_device_noalloc (every intermediate in the library's fixed
device pool) against rive_cuda_flush_device on the golden captures that fit
its limits. Both run the same kernels on the same records, so two calls in a
row must each give exactly the context path's image, bit for bit: a stale
value left in the reused pool by an earlier call would show as a difference.
The second call must leave the device's free memory unchanged. Flushes
beyond the pool's size limits are refused on the host before anything is
launched; one whose tile bins outgrow the pool is refused after set-up, with
the target untouched.

Collected last on purpose, so it also runs after every other GPU test has used
the device in this process.
"""
import numpy as np
import pytest

from conftest import device_buffers, golden_names, load_golden, load_package

load_package()

LIMIT_W = 1024
LIMIT_TESS_ROWS = 32
LIMIT_GRAD_ROWS = 64
LIMIT_BIN_ENTRIES = 1 << 20


def _fits(cap):
    return (cap.width <= LIMIT_W and cap.height <= LIMIT_W and
            all(f.desc["tess_data_height"] <= LIMIT_TESS_ROWS and
                f.desc["grad_data_height"] <= LIMIT_GRAD_ROWS for f in cap.flushes))


def _fans_only(cap):
    # The no-allocation path draws midpoint-fan batches only (no interior
    # triangulation, no center-AA fans of feathered fills) and no images.
    return not cap.textures and not any(
        f.desc["has_triangle_vertices"] or (f.batches[:, 0] != 0).any() for f in cap.flushes)


def _context_image(cap, bufs, stream):
    import torch
    from rive_runtime_gb300 import rive_cuda
    ctx = rive_cuda.Context(0)
    try:
        t = torch.zeros((cap.height, cap.width, 4), dtype=torch.uint8, device="cuda")
        for f in cap.flushes:
            ctx.flush_device(f, bufs, t.data_ptr(), stream)
        ctx.sync(stream)
        torch.cuda.synchronize()
        return t.cpu().numpy(), ctx.stats()
    finally:
        ctx.close()


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in golden_names()
                                  if _fits(load_golden(n)[0]) and _fans_only(load_golden(n)[0])])
def test_noalloc_matches_flush_device_twice(name):
    import torch
    from rive_runtime_gb300 import rive_cuda
    cap, _ = load_golden(name)
    bufs, keep = device_buffers(cap)
    stream = torch.cuda.current_stream().cuda_stream
    want, _ = _context_image(cap, bufs, stream)
    shape = (cap.height, cap.width, 4)
    for call in range(2):
        got_t = torch.zeros(shape, dtype=torch.uint8, device="cuda")
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        for f in cap.flushes:
            rive_cuda.flush_device_noalloc(f, bufs, got_t.data_ptr(), stream)
        torch.cuda.synchronize()
        free_after = torch.cuda.mem_get_info()[0]
        if call == 1:
            # The first call on a device may load the module (and with it
            # the pool); later calls allocate nothing.
            assert free_after == free_before, (name, free_before, free_after)
        assert np.array_equal(got_t.cpu().numpy(), want), (name, call)
    del keep


@pytest.mark.gpu
def test_noalloc_refuses_flushes_beyond_its_limits():
    import torch
    from rive_runtime_gb300 import rive_cuda
    big = [n for n in golden_names()
           if not _fits(load_golden(n)[0]) and _fans_only(load_golden(n)[0])]
    assert big, "expected a golden capture beyond the no-allocation limits"
    cap, _ = load_golden(big[0])
    bufs, keep = device_buffers(cap)
    target = torch.full((cap.height, cap.width, 4), 7, dtype=torch.uint8, device="cuda")
    with pytest.raises(rive_cuda.RiveCudaError, match="no-allocation limit"):
        rive_cuda.flush_device_noalloc(cap.flushes[0], bufs, target.data_ptr(),
                                       torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert bool((target == 7).all()), "a refused flush must not write the target"
    del keep


@pytest.mark.gpu
def test_noalloc_refuses_the_feather_atlas():
    """The atlas's intermediates have no room in the fixed pool: a flush that
    renders one is refused before launch, the target untouched."""
    import torch
    from rive_runtime_gb300 import rive_cuda
    cap, _ = load_golden("feather_atlas_s35")
    assert cap.flushes[0].has_atlas
    bufs, keep = device_buffers(cap)
    target = torch.full((cap.height, cap.width, 4), 7, dtype=torch.uint8, device="cuda")
    with pytest.raises(rive_cuda.RiveCudaError, match="feather atlas"):
        rive_cuda.flush_device_noalloc(cap.flushes[0], bufs, target.data_ptr(),
                                       torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert bool((target == 7).all())
    del keep


def _star_scene(n_paths):
    """n_paths star polygons {40/17} of radius 380-500 px around the middle
    of a 1024x1024 canvas: few tessellation vertices (one segment per
    straight edge), but long edges and fan triangles that each cross hundreds
    of tiles."""
    import math
    from rive_runtime_gb300 import scene
    rng = np.random.default_rng(9)
    sc = scene.Scene(1024, 1024, clear_color=0xFFFFFFFF)
    k, step = 40, 17
    for _ in range(n_paths):
        c = rng.uniform(400, 624, 2)
        r = rng.uniform(380, 500)
        ang = rng.uniform(0, 2 * math.pi) + 2 * math.pi * ((np.arange(k) * step) % k) / k
        pts = np.stack([c[0] + r * np.cos(ang), c[1] + r * np.sin(ang)], 1).astype(np.float32)
        verbs = [scene.VERB_MOVE] + [scene.VERB_LINE] * (k - 1) + [scene.VERB_CLOSE]
        pi = sc.add_path(scene.Path(verbs, pts, scene.FILL_NONZERO))
        qi = sc.add_paint(scene.Paint(style=scene.STYLE_FILL,
                                      color=scene.color_int(*rng.uniform(0, 1, 3), 1.0)))
        sc.cmd(scene.CMD_DRAW_PATH, pi, qi)
    return sc


@pytest.mark.gpu
def test_noalloc_refuses_a_bin_overflow_after_setup():
    """A 1024x1024 frame of 200 star polygons fits every size limit known
    before launch (16 tessellation rows, 4,000 patches), but its triangles
    overlap more than 2^20 (tile, triangle) pairs: the call stops after
    set-up and leaves the target untouched."""
    import torch
    from rive_runtime_gb300 import rive_cuda
    from inputgen import planner
    cap = planner.plan(_star_scene(200).to_bytes())
    assert _fits(cap) and _fans_only(cap) and len(cap.flushes) == 1
    bufs, keep = device_buffers(cap)
    stream = torch.cuda.current_stream().cuda_stream
    target = torch.full((cap.height, cap.width, 4), 7, dtype=torch.uint8, device="cuda")
    with pytest.raises(rive_cuda.RiveCudaError, match="bin entries exceed the no-allocation"):
        rive_cuda.flush_device_noalloc(cap.flushes[0], bufs, target.data_ptr(), stream)
    torch.cuda.synchronize()
    assert bool((target == 7).all()), "a refused flush must not write the target"
    # A following call that fits still renders.
    small, _ = load_golden(next(n for n in golden_names()
                                if _fits(load_golden(n)[0]) and _fans_only(load_golden(n)[0])))
    sbufs, skeep = device_buffers(small)
    want, _ = _context_image(small, sbufs, stream)
    got = torch.zeros((small.height, small.width, 4), dtype=torch.uint8, device="cuda")
    rive_cuda.flush_device_noalloc(small.flushes[0], sbufs, got.data_ptr(), stream)
    torch.cuda.synchronize()
    assert np.array_equal(got.cpu().numpy(), want)
    del keep, skeep


def test_noalloc_rejects_null_arguments_without_a_gpu_call():
    import ctypes
    from rive_runtime_gb300 import rive_cuda
    lib = rive_cuda.load()
    err = ctypes.create_string_buffer(256)
    assert lib.rive_cuda_flush_device_noalloc(None, None, None, None, err, 256) == 1
    assert err.value  # a message names the problem
