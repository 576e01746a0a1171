"""rive_cuda_flush_device_noalloc (every intermediate in the library's fixed
device pool) against rive_cuda_flush_device on the golden captures that fit its
limits: two calls in a row must each give the image the context path gives,
within the image tolerance of the parity tests (2/255 per channel on >= 99.9%
of pixels, 8/255 everywhere). Flushes beyond the pool's limits are refused on
the host before anything is launched.

Collected last on purpose, so it also runs after every other GPU test has used
the device in this process.
"""
import numpy as np
import pytest

from conftest import golden_names, load_golden, load_package

load_package()

LIMIT_W = 1024
LIMIT_TESS_ROWS = 32


def _fits(cap):
    return (cap.width <= LIMIT_W and cap.height <= LIMIT_W and
            all(f.desc["tess_data_height"] <= LIMIT_TESS_ROWS for f in cap.flushes))


def _fans_only(cap):
    # The no-allocation path draws midpoint-fan batches only (no interior
    # triangulation, no center-AA fans of feathered fills).
    return not any(f.desc["has_triangle_vertices"] or (f.batches[:, 0] != 0).any()
                   for f in cap.flushes)


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


def _within_tolerance(got, want):
    d = np.abs(got.astype(np.int16) - want.astype(np.int16)).max(axis=2)
    return float((d <= 2).mean()) >= 0.999 and int(d.max()) <= 8


@pytest.mark.gpu
@pytest.mark.parametrize("name", [n for n in golden_names()
                                  if _fits(load_golden(n)[0]) and _fans_only(load_golden(n)[0])])
def test_noalloc_matches_flush_device_twice(name):
    import torch
    from rive_runtime_gb300 import rive_cuda
    cap, _ = load_golden(name)
    bufs, keep = _device_buffers(cap)
    stream = torch.cuda.current_stream().cuda_stream
    shape = (cap.height, cap.width, 4)

    ctx = rive_cuda.Context(0)
    try:
        want_t = torch.zeros(shape, dtype=torch.uint8, device="cuda")
        for f in cap.flushes:
            ctx.flush_device(f, bufs, want_t.data_ptr(), stream)
        ctx.sync(stream)
        torch.cuda.synchronize()
        want = want_t.cpu().numpy()
    finally:
        ctx.close()

    for call in range(2):
        got_t = torch.zeros(shape, dtype=torch.uint8, device="cuda")
        for f in cap.flushes:
            rive_cuda.flush_device_noalloc(f, bufs, got_t.data_ptr(), stream)
        torch.cuda.synchronize()
        got = got_t.cpu().numpy()
        assert _within_tolerance(got, want), (name, call)
    del keep


@pytest.mark.gpu
def test_noalloc_refuses_flushes_beyond_its_limits():
    import torch
    from rive_runtime_gb300 import rive_cuda
    big = [n for n in golden_names()
           if not _fits(load_golden(n)[0]) and _fans_only(load_golden(n)[0])]
    assert big, "expected a golden capture beyond the no-allocation limits"
    cap, _ = load_golden(big[0])
    bufs, keep = _device_buffers(cap)
    target = torch.full((cap.height, cap.width, 4), 7, dtype=torch.uint8, device="cuda")
    with pytest.raises(rive_cuda.RiveCudaError, match="no-allocation limit"):
        rive_cuda.flush_device_noalloc(cap.flushes[0], bufs, target.data_ptr(),
                                       torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    assert bool((target == 7).all()), "a refused flush must not write the target"
    del keep


def test_noalloc_rejects_null_arguments_without_a_gpu_call():
    import ctypes
    from rive_runtime_gb300 import rive_cuda
    lib = rive_cuda.load()
    err = ctypes.create_string_buffer(256)
    assert lib.rive_cuda_flush_device_noalloc(None, None, None, None, err, 256) == 1
    assert err.value  # a message names the problem
