"""TEST INFRASTRUCTURE: ctypes binding of the CPU oracle (passes.c) and of the
reference front-end replay (oracle/_ref/ref_capture, built here only).

Only tests, the smoke check and the benchmark's CPU-baseline leg import this
module, and only to check or time against; the product never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "_build", "liboracle_passes.so")
REF_CAPTURE = os.path.join(HERE, "_ref", "ref_capture")
ADAPTER_CAPTURE = os.path.join(HERE, "_ref", "adapter_capture")
# The reference sources, where they exist (this build machine only):
# RIVE_REFERENCE_DIR, or the default checkout location.
REFERENCE_SOURCES = os.environ.get("RIVE_REFERENCE_DIR", "/root/reference")

BUFFER_NAMES = ("flush_uniforms", "paths", "paints", "paint_aux", "contours",
                "grad_spans", "tess_spans", "triangles", "image_draws")


class FlushDesc(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint32) for n in (
        "render_target_width", "render_target_height", "interlock_mode",
        "color_load_action", "color_clear_value")] + [
        ("update_bounds", ctypes.c_int32 * 4)] + [
        (n, ctypes.c_uint32) for n in (
            "combined_shader_features", "dither_mode",
            "flush_uniform_offset_bytes", "path_count", "first_path",
            "first_paint", "first_paint_aux", "contour_count", "first_contour",
            "grad_span_count", "first_grad_span", "tess_span_count",
            "first_tess_span", "grad_data_height", "tess_data_height",
            "grad_texture_height", "wireframe", "clockwise_fill_override",
            "has_triangle_vertices",
            "draw_batch_count")] + [("draw_batches", ctypes.c_void_p)] + [
        (n, ctypes.c_uint32) for n in (
            "atlas_texture_width", "atlas_texture_height", "atlas_content_width",
            "atlas_content_height", "atlas_fill_batch_count",
            "atlas_stroke_batch_count")] + [("atlas_batches", ctypes.c_void_p),
                                            ("batch_images", ctypes.c_void_p),
                                            ("batch_meshes", ctypes.c_void_p)]


class OracleTexture(ctypes.Structure):
    """oracle_texture (passes.h)."""
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32),
                ("levels", ctypes.c_uint32), ("rgba", ctypes.c_void_p),
                ("mips", ctypes.c_void_p), ("off", ctypes.c_uint32 * 16)]


class BatchImage(ctypes.Structure):
    """rive_cuda_batch_image, its texture pointing at an OracleTexture."""
    _fields_ = [("texture", ctypes.c_void_p), ("sampler_key", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class OracleRenderBuffer(ctypes.Structure):
    """oracle_render_buffer (passes.h)."""
    _fields_ = [("data", ctypes.c_void_p), ("bytes", ctypes.c_size_t)]


class BatchMesh(ctypes.Structure):
    """rive_cuda_batch_mesh, its buffers pointing at OracleRenderBuffers."""
    _fields_ = [("vertices", ctypes.c_void_p), ("uvs", ctypes.c_void_p),
                ("indices", ctypes.c_void_p), ("index_count", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class OracleBuffers(ctypes.Structure):
    _fields_ = []
    for _n in BUFFER_NAMES:
        _fields_ += [(_n, ctypes.c_void_p), (_n + "_bytes", ctypes.c_size_t)]


def build():
    subprocess.check_call(["make", "-s", "-C", HERE, "passes"])


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        for name in ("oracle_color_ramps", "oracle_tessellate", "oracle_draw",
                     "oracle_flush", "oracle_tessellate_f64", "oracle_atlas",
                     "oracle_texture_prepare"):
            getattr(_lib, name).restype = ctypes.c_int
        _lib.oracle_f32_to_f16.restype = ctypes.c_uint16
        _lib.oracle_f32_to_f16.argtypes = [ctypes.c_float]
        _lib.oracle_f16_to_f32.restype = ctypes.c_float
        _lib.oracle_f16_to_f32.argtypes = [ctypes.c_uint16]
        _lib.oracle_mesh_mip_level.restype = ctypes.c_int
        _lib.oracle_mesh_mip_level.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_uint32]
    return _lib


def make_desc(flush):
    """rive_cuda_flush_desc for one capture.Flush (keeps the batch array alive)."""
    d = FlushDesc()
    for k, v in flush.desc.items():
        if k.startswith("ub"):
            d.update_bounds[int(k[2])] = v
        elif k != "draw_batch_count":
            setattr(d, k, v)
    batches = np.ascontiguousarray(flush.batches, dtype=np.uint32)
    d.draw_batch_count = len(batches)
    d.draw_batches = batches.ctypes.data if len(batches) else None
    # rive_cuda_atlas_batch: u16 scissor[4], u32 patch_count, u32 base_patch
    # (the capture's (n, 4) uint32 rows have the same bytes).
    atlas = np.ascontiguousarray(getattr(flush, "atlas", np.zeros((0, 4), np.uint32)),
                                 dtype=np.uint32).reshape(-1, 4)
    d.atlas_batches = atlas.ctypes.data if len(atlas) else None
    images = textures = None
    if getattr(flush, "has_images", False):
        textures = _textures(flush.textures)
        images = (BatchImage * len(batches))()
        for i, (tex, key) in enumerate(np.asarray(flush.images, dtype=np.uint32)):
            if tex != 0xFFFFFFFF:
                images[i].texture = ctypes.addressof(textures[int(tex)][0])
                images[i].sampler_key = int(key)
        d.batch_images = ctypes.addressof(images)
    meshes = rbufs = None
    if getattr(flush, "has_meshes", False):
        rbufs = [(OracleRenderBuffer(ctypes.cast(ctypes.c_char_p(b.data), ctypes.c_void_p).value,
                                     len(b.data)), b) for b in flush.render_buffers]
        meshes = (BatchMesh * len(batches))()
        for i, (vb, ub, ib, n) in enumerate(np.asarray(flush.meshes, dtype=np.uint32)):
            if vb != 0xFFFFFFFF:
                meshes[i].vertices = ctypes.addressof(rbufs[int(vb)][0])
                meshes[i].uvs = ctypes.addressof(rbufs[int(ub)][0])
                meshes[i].indices = ctypes.addressof(rbufs[int(ib)][0])
                meshes[i].index_count = int(n)
        d.batch_meshes = ctypes.addressof(meshes)
    return d, (batches, atlas, images, textures, meshes, rbufs)


# Prepared oracle textures (mip chains made by oracle_texture_prepare), kept
# per capture.Texture object.
_TEXTURES = {}


def _textures(texs):
    out = []
    for t in texs:
        key = id(t)
        if key not in _TEXTURES:
            data = np.frombuffer(t.rgba, np.uint8).copy()
            ot = OracleTexture(t.width, t.height, t.mip_levels,
                               data.ctypes.data_as(ctypes.c_void_p).value, None)
            _check(lib().oracle_texture_prepare(ctypes.byref(ot)), "texture_prepare")
            _TEXTURES[key] = (ot, data, t)
        out.append(_TEXTURES[key])
    return out


def make_buffers(cap):
    keep = []
    b = OracleBuffers()
    for n in BUFFER_NAMES:
        data = cap.buffers.get(n, b"")
        arr = np.frombuffer(data, dtype=np.uint8).copy() if data else np.zeros(16, np.uint8)
        keep.append(arr)
        setattr(b, n, arr.ctypes.data)
        setattr(b, n + "_bytes", len(data))
    return b, keep


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed with {rc}")


def color_ramps(cap, fi=0):
    f = cap.flushes[fi]
    d, _k1 = make_desc(f)
    b, _k2 = make_buffers(cap)
    h = max(int(f.desc["grad_data_height"]), 1)
    out = np.zeros((h, 512, 4), np.uint8)
    _check(lib().oracle_color_ramps(ctypes.byref(d), ctypes.byref(b),
                                    out.ctypes.data_as(ctypes.c_void_p)), "color ramps")
    return out


def tessellate(cap, fi=0):
    f = cap.flushes[fi]
    d, _k1 = make_desc(f)
    b, _k2 = make_buffers(cap)
    h = max(int(f.desc["tess_data_height"]), 1)
    out = np.zeros((h * 2048, 4), np.uint32)
    _check(lib().oracle_tessellate(ctypes.byref(d), ctypes.byref(b),
                                   out.ctypes.data_as(ctypes.c_void_p)), "tessellate")
    return out


def tessellate_f64(cap, fi=0):
    f = cap.flushes[fi]
    d, _k1 = make_desc(f)
    b, _k2 = make_buffers(cap)
    h = max(int(f.desc["tess_data_height"]), 1)
    xy = np.zeros((h * 2048, 2), np.float64)
    flags = np.zeros(h * 2048, np.uint32)
    _check(lib().oracle_tessellate_f64(ctypes.byref(d), ctypes.byref(b),
                                       xy.ctypes.data_as(ctypes.c_void_p),
                                       flags.ctypes.data_as(ctypes.c_void_p)),
           "tessellate_f64")
    return xy, flags


def atlas(cap, fi=0, threads=0):
    """The feather atlas logical flush `fi` renders (fp16 texels as float32,
    atlas_content_height x atlas_content_width)."""
    f = cap.flushes[fi]
    d, _k1 = make_desc(f)
    b, _k2 = make_buffers(cap)
    h, w = int(f.desc["atlas_content_height"]), int(f.desc["atlas_content_width"])
    out = np.zeros((max(h, 1), max(w, 1)), np.uint16)
    _check(lib().oracle_atlas(ctypes.byref(d), ctypes.byref(b),
                              out.ctypes.data_as(ctypes.c_void_p), int(threads)), "atlas")
    return out[:h, :w].view(np.float16).astype(np.float32)


def render(cap, threads=0, fb=None):
    """Runs every logical flush of the capture in order; returns HxWx4 RGBA8."""
    if fb is None:
        fb = np.zeros((cap.height, cap.width, 4), np.uint8)
    b, _keep = make_buffers(cap)
    for f in cap.flushes:
        d, _k = make_desc(f)
        _check(lib().oracle_flush(ctypes.byref(d), ctypes.byref(b),
                                  fb.ctypes.data_as(ctypes.c_void_p), int(threads)),
               "flush")
    return fb


def render_flush(cap, fi, fb, threads=0):
    """Runs logical flush `fi` of the capture onto `fb` (HxWx4 RGBA8)."""
    b, _keep = make_buffers(cap)
    d, _k = make_desc(cap.flushes[fi])
    _check(lib().oracle_flush(ctypes.byref(d), ctypes.byref(b),
                              fb.ctypes.data_as(ctypes.c_void_p), int(threads)), "flush")
    return fb


def mesh_mip_level(rho2, bias=-0.5, levels=16):
    """The mip level an image-mesh triangle samples (passes.c mesh_mip_level)."""
    return lib().oracle_mesh_mip_level(float(rho2), float(bias), int(levels))


def last_stats():
    t = ctypes.c_uint64()
    fr = ctypes.c_uint64()
    lib().oracle_last_stats(ctypes.byref(t), ctypes.byref(fr))
    return t.value, fr.value


def feather_table():
    """The oracle's 512-entry fp16 feather table (uint16 bits)."""
    out = np.zeros(512, np.uint16)
    lib().oracle_feather_table(out.ctypes.data_as(ctypes.c_void_p))
    return out


def inverse_feather_table():
    """The oracle's 512-entry fp16 inverse feather table (uint16 bits)."""
    out = np.zeros(512, np.uint16)
    lib().oracle_inverse_feather_table(out.ctypes.data_as(ctypes.c_void_p))
    return out


def f32_to_f16(x):
    return lib().oracle_f32_to_f16(float(x))


def f16_to_f32(h):
    return lib().oracle_f16_to_f32(int(h))


def reference_available():
    return os.path.isdir(REFERENCE_SOURCES)


def _make_env():
    return dict(os.environ, REF=REFERENCE_SOURCES)


def build_reference():
    subprocess.check_call(["make", "-s", "-j8", "-C", HERE, "ref"], env=_make_env())


CMDBUF_CAPTURE = os.path.join(HERE, "_ref", "cmdbuf_capture")


def build_cmdbuf_tool() -> str:
    """Builds (if needed) the reference's deferred command recorder/replayer
    tool (oracle/capture/cmdbuf_capture.cpp); returns its path."""
    subprocess.check_call(["make", "-s", "-j8", "-C", HERE, "cmdbuf"], env=_make_env())
    return CMDBUF_CAPTURE


def cmdbuf_record(scene_bytes: bytes) -> bytes:
    """The reference's DeferredFactory recording of a scene (.rcb bytes)."""
    tool = build_cmdbuf_tool()
    with tempfile.TemporaryDirectory() as td:
        sp, rp = os.path.join(td, "scene.bin"), os.path.join(td, "s.rcb")
        with open(sp, "wb") as f:
            f.write(scene_bytes)
        subprocess.check_call([tool, "record", sp, rp])
        with open(rp, "rb") as f:
            return f.read()


def cmdbuf_replay(rcb_bytes: bytes) -> bytes:
    """The reference's replayRenderCommands of a stored stream, captured."""
    tool = build_cmdbuf_tool()
    with tempfile.TemporaryDirectory() as td:
        rp, cp = os.path.join(td, "s.rcb"), os.path.join(td, "capture.bin")
        with open(rp, "wb") as f:
            f.write(rcb_bytes)
        subprocess.check_call([tool, "replay", rp, cp])
        with open(cp, "rb") as f:
            return f.read()


def _run_capture(tool: str, scene_bytes: bytes) -> bytes:
    with tempfile.TemporaryDirectory() as td:
        sp = os.path.join(td, "scene.bin")
        cp = os.path.join(td, "capture.bin")
        with open(sp, "wb") as f:
            f.write(scene_bytes)
        subprocess.check_call([tool, sp, cp])
        with open(cp, "rb") as f:
            return f.read()


def reference_capture(scene_bytes: bytes) -> bytes:
    """Runs the reference front end on a scene; returns the capture bytes."""
    if not os.path.exists(REF_CAPTURE):
        build_reference()
    return _run_capture(REF_CAPTURE, scene_bytes)


def adapter_capture(scene_bytes: bytes) -> bytes:
    """Runs the reference front end into the product's RenderContextCUDAImpl
    over the recording C ABI; returns what reached the ABI as a capture."""
    subprocess.check_call(["make", "-s", "-j8", "-C", HERE, "adapter"], env=_make_env())
    return _run_capture(ADAPTER_CAPTURE, scene_bytes)
