"""Shared test set-up: the `gpu` marker and the package loader.

The package directory is named `rive-runtime_gb300` (not an identifier), so it
is loaded under the module name `rive_runtime_gb300`.
"""
import importlib.util
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(REPO, "tests", "golden")


def load_package():
    if "rive_runtime_gb300" in sys.modules:
        return sys.modules["rive_runtime_gb300"]
    root = os.path.join(REPO, "rive-runtime_gb300")
    spec = importlib.util.spec_from_file_location(
        "rive_runtime_gb300", os.path.join(root, "__init__.py"),
        submodule_search_locations=[root])
    mod = importlib.util.module_from_spec(spec)
    sys.modules["rive_runtime_gb300"] = mod
    spec.loader.exec_module(mod)
    return mod


load_package()
if os.path.join(REPO, "oracle") not in sys.path:
    sys.path.insert(0, os.path.join(REPO, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_names():
    return sorted(f[:-4] for f in os.listdir(GOLDEN) if f.endswith(".cap"))


def load_golden(name):
    from rive_runtime_gb300 import capture
    with open(os.path.join(GOLDEN, name + ".cap"), "rb") as f:
        cap = capture.parse(f.read())
    with open(os.path.join(GOLDEN, name + ".scene"), "rb") as f:
        scene_bytes = f.read()
    return cap, scene_bytes


def tess_written(cap, fi):
    """Texels of the tessellation texture that logical flush fi writes: each
    TessVertexSpan covers [x0, x1) of row y and, mirrored, [rx0, rx1) of row
    ry (gpu.hpp:291-376); both passes skip a NaN or out-of-range row and an
    empty range. Texels outside them keep whatever an earlier flush left."""
    import numpy as np
    d = cap.flushes[fi].desc
    h = max(int(d["tess_data_height"]), 1)
    mask = np.zeros(h * 2048, bool)
    spans = np.frombuffer(cap.buffers.get("tess_spans", b""), np.uint32).reshape(-1, 16)
    spans = spans[d["first_tess_span"]:d["first_tess_span"] + d["tess_span_count"]]
    for yw, xw in ((10, 12), (11, 13)):
        y = spans[:, yw].view(np.float32)
        x0 = (spans[:, xw].astype(np.int64) << 48 >> 48).astype(np.int64)
        x1 = (spans[:, xw].view(np.int32) >> 16).astype(np.int64)
        ok = ~np.isnan(y) & (x0 != x1) & (y >= 0) & (y < h)
        for yy, a, b in zip(y[ok].astype(np.int64), x0[ok], x1[ok]):
            lo, hi = max(min(a, b), 0), min(max(a, b), 2048)
            if lo < hi:
                mask[yy * 2048 + lo: yy * 2048 + hi] = True
    return mask


def device_buffers(cap):
    """The capture's record buffers as device tensors, as
    rive_cuda_device_buffers (keep the returned tensors alive)."""
    import numpy as np
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


def flush_waves(caps, bufs, targets):
    """Wave i holds logical flush i of every frame that has one: the flushes
    of one wave are independent (distinct targets), while a frame's later
    flushes load what its earlier ones wrote, so waves run in order."""
    n = max(len(c.flushes) for c in caps)
    return [[(c.flushes[i], b, t.data_ptr()) for c, b, t in zip(caps, bufs, targets)
             if i < len(c.flushes)] for i in range(n)]


def render_one_by_one(ctx, caps, bufs, stream):
    """Every frame flushed one logical flush at a time through
    rive_cuda_flush_device; returns the images."""
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
