"""ctypes binding of the C ABI in include/rive_cuda.h (librive_cuda.so).

This is the Python face of the drop-in backend: the same calls a
RenderContextImpl makes (resize/map/unmap per record buffer, then one flush per
logical flush), plus render-target read-back. The library is built in-tree by
``build.py``; importing this module on a machine without it raises, so no code
path can silently fall back to the CPU.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

from . import build as _build
from .capture import BUFFER_NAMES

LIB_PATH = _build.LIB
HEADER = os.path.join(_build.REPO, "include", "rive_cuda.h")

OK = 0
STAGES = ("color_ramp", "tessellate", "patch_setup", "bin", "sort", "raster")
BUFFER_KINDS = {n: i for i, n in enumerate(BUFFER_NAMES)}


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


class BatchImage(ctypes.Structure):
    """rive_cuda_batch_image."""
    _fields_ = [("texture", ctypes.c_void_p), ("sampler_key", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class BatchMesh(ctypes.Structure):
    """rive_cuda_batch_mesh."""
    _fields_ = [("vertices", ctypes.c_void_p), ("uvs", ctypes.c_void_p),
                ("indices", ctypes.c_void_p), ("index_count", ctypes.c_uint32),
                ("reserved", ctypes.c_uint32)]


class DeviceBuffers(ctypes.Structure):
    # rive_cuda_device_buffers (triangles = triangle_vertices).
    _fields_ = [(n, ctypes.c_void_p) for n in (
        "flush_uniforms", "paths", "paints", "paint_aux", "contours",
        "grad_spans", "tess_spans", "triangles", "image_draws")]


class BatchFlush(ctypes.Structure):
    _fields_ = [("desc", ctypes.c_void_p), ("buffers", DeviceBuffers),
                ("target_pixels_device", ctypes.c_void_p)]


class FlushStats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "tess_vertices", "patches", "triangles", "bin_entries", "tiles",
        "kernel_launches", "winding_entries")]


class RiveCudaError(RuntimeError):
    pass


_lib = None


def exported_functions():
    """Names of the functions include/rive_cuda.h declares."""
    with open(HEADER) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(rive_cuda_[a-z0-9_]+)\s*\(", text)))


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"librive_cuda.so is not built ({LIB_PATH}); run __graft_entry__.build()")
    lib = ctypes.CDLL(LIB_PATH)
    vp, sz, u32, i32 = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_uint32, ctypes.c_int
    sig = {
        "rive_cuda_context_create": (i32, [i32, ctypes.POINTER(vp)]),
        "rive_cuda_context_destroy": (None, [vp]),
        "rive_cuda_last_error": (i32, [vp, ctypes.c_char_p, sz]),
        "rive_cuda_resize_buffer": (i32, [vp, i32, sz]),
        "rive_cuda_map_buffer": (vp, [vp, i32, sz]),
        "rive_cuda_unmap_buffer": (i32, [vp, i32, sz]),
        "rive_cuda_resize_gradient_texture": (i32, [vp, u32, u32]),
        "rive_cuda_resize_tessellation_texture": (i32, [vp, u32, u32]),
        "rive_cuda_render_target_create": (i32, [vp, u32, u32, ctypes.POINTER(vp)]),
        "rive_cuda_render_target_destroy": (None, [vp, vp]),
        "rive_cuda_render_target_device_ptr": (vp, [vp]),
        "rive_cuda_render_target_read": (i32, [vp, vp, vp, vp]),
        "rive_cuda_render_target_read_async": (i32, [vp, vp, vp, vp]),
        "rive_cuda_flush": (i32, [vp, ctypes.POINTER(FlushDesc), vp, vp]),
        "rive_cuda_flush_device": (i32, [vp, ctypes.POINTER(FlushDesc),
                                         ctypes.POINTER(DeviceBuffers), vp, vp]),
        "rive_cuda_flush_batch": (i32, [vp, ctypes.POINTER(BatchFlush), u32, vp]),
        "rive_cuda_graph_create": (i32, [vp, ctypes.POINTER(BatchFlush), u32, u32,
                                         ctypes.POINTER(vp)]),
        "rive_cuda_graph_launch": (i32, [vp, vp]),
        "rive_cuda_graph_check": (i32, [vp, vp]),
        "rive_cuda_graph_stats": (i32, [vp, ctypes.POINTER(FlushStats)]),
        "rive_cuda_graph_destroy": (None, [vp]),
        "rive_cuda_flush_device_noalloc": (i32, [ctypes.POINTER(FlushDesc),
                                                 ctypes.POINTER(DeviceBuffers), vp, vp,
                                                 ctypes.c_char_p, sz]),
        "rive_cuda_sync": (i32, [vp, vp]),
        "rive_cuda_read_tess_texture": (i32, [vp, vp, sz]),
        "rive_cuda_read_grad_texture": (i32, [vp, vp, sz]),
        "rive_cuda_read_atlas_texture": (i32, [vp, vp, sz]),
        "rive_cuda_texture_create": (i32, [vp, u32, u32, u32, vp, ctypes.POINTER(vp)]),
        "rive_cuda_texture_destroy": (None, [vp, vp]),
        "rive_cuda_texture_read": (i32, [vp, vp, u32, vp, sz]),
        "rive_cuda_render_buffer_create": (i32, [vp, u32, sz, ctypes.POINTER(vp)]),
        "rive_cuda_render_buffer_write": (i32, [vp, vp, sz, vp, sz]),
        "rive_cuda_render_buffer_destroy": (None, [vp, vp]),
        "rive_cuda_last_flush_stats": (i32, [vp, ctypes.POINTER(FlushStats)]),
        "rive_cuda_set_profiling": (i32, [vp, i32]),
        "rive_cuda_set_raster_config": (i32, [vp, i32, i32]),
        "rive_cuda_set_winding_tiles": (i32, [vp, i32]),
        "rive_cuda_set_raster_queue": (i32, [vp, i32]),
        "rive_cuda_set_bin_speculation": (i32, [vp, i32]),
        "rive_cuda_get_bin_speculation": (i32, [vp, ctypes.POINTER(ctypes.c_int)]),
        "rive_cuda_get_raster_queue": (i32, [vp, ctypes.POINTER(ctypes.c_int)]),
        "rive_cuda_eval_tessellation_math": (i32, [i32, vp, vp, sz]),
        "rive_cuda_get_winding_tiles": (i32, [vp, ctypes.POINTER(ctypes.c_int)]),
        "rive_cuda_feather_table": (i32, [vp]),
        "rive_cuda_inverse_feather_table": (i32, [vp]),
        "rive_cuda_get_raster_config": (i32, [vp, ctypes.POINTER(ctypes.c_int),
                                              ctypes.POINTER(ctypes.c_int)]),
        "rive_cuda_profile_collect": (i32, [vp, ctypes.POINTER(ctypes.c_double),
                                            ctypes.POINTER(ctypes.c_uint64)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def make_desc(flush, textures=None, buffers=None):
    """rive_cuda_flush_desc for one capture.Flush. `textures` maps the
    capture's texture indices to rive_cuda_texture handles (needed when a
    batch draws an image), `buffers` its render-buffer indices to
    rive_cuda_render_buffer handles (needed when a batch draws an image
    mesh). Returns (desc, arrays to keep alive)."""
    d = FlushDesc()
    for k, v in flush.desc.items():
        if k.startswith("ub"):
            d.update_bounds[int(k[2])] = v
        elif k != "draw_batch_count":
            setattr(d, k, int(v))
    batches = np.ascontiguousarray(flush.batches, dtype=np.uint32)
    d.draw_batch_count = len(batches)
    d.draw_batches = batches.ctypes.data if len(batches) else None
    # rive_cuda_atlas_batch: u16 scissor[4], u32 patch_count, u32 base_patch
    # (the capture's (n, 4) uint32 rows have the same bytes).
    atlas = np.ascontiguousarray(getattr(flush, "atlas", np.zeros((0, 4), np.uint32)),
                                 dtype=np.uint32).reshape(-1, 4)
    d.atlas_batches = atlas.ctypes.data if len(atlas) else None
    images = None
    if getattr(flush, "has_images", False):
        if textures is None:
            raise RiveCudaError("the flush draws images: pass its textures")
        images = (BatchImage * len(batches))()
        for i, (tex, key) in enumerate(np.asarray(flush.images, dtype=np.uint32)):
            if tex != 0xFFFFFFFF:
                images[i].texture = textures[int(tex)]
                images[i].sampler_key = int(key)
        d.batch_images = ctypes.addressof(images)
    meshes = None
    if getattr(flush, "has_meshes", False):
        if buffers is None:
            raise RiveCudaError("the flush draws image meshes: pass its render buffers")
        meshes = (BatchMesh * len(batches))()
        for i, (vb, ub, ib, n) in enumerate(np.asarray(flush.meshes, dtype=np.uint32)):
            if vb != 0xFFFFFFFF:
                meshes[i].vertices = buffers[int(vb)]
                meshes[i].uvs = buffers[int(ub)]
                meshes[i].indices = buffers[int(ib)]
                meshes[i].index_count = int(n)
        d.batch_meshes = ctypes.addressof(meshes)
    return d, (batches, atlas, images, meshes)


def feather_table():
    """The fp16 bits of the library's feather table (512 entries)."""
    out = np.zeros(512, np.uint16)
    rc = load().rive_cuda_feather_table(out.ctypes.data_as(ctypes.c_void_p))
    if rc != OK:
        raise RiveCudaError(f"feather_table: status {rc}")
    return out


def inverse_feather_table():
    """The fp16 bits of the library's inverse feather table (512 entries)."""
    out = np.zeros(512, np.uint16)
    rc = load().rive_cuda_inverse_feather_table(out.ctypes.data_as(ctypes.c_void_p))
    if rc != OK:
        raise RiveCudaError(f"inverse_feather_table: status {rc}")
    return out


def flush_device_noalloc(flush, bufs: DeviceBuffers, target_ptr: int, stream=None):
    """rive_cuda_flush_device_noalloc: one flush of a small frame with every
    intermediate in the library's fixed device pool (no context, no
    allocation). Synchronous; raises RiveCudaError with the library's message."""
    lib = load()
    d, keep = make_desc(flush)
    err = ctypes.create_string_buffer(512)
    rc = lib.rive_cuda_flush_device_noalloc(ctypes.byref(d), ctypes.byref(bufs),
                                            ctypes.c_void_p(target_ptr), stream, err, 512)
    del keep
    if rc != OK:
        raise RiveCudaError(f"flush_device_noalloc: status {rc}: {err.value.decode()}")


TESS_MATH_LAYOUT = {0: (2, 1), 1: (8, 2), 2: (10, 1), 3: (9, 2), 4: (12, 1), 5: (8, 4),
                    10: (1, 1), 11: (1, 1), 12: (1, 1), 13: (1, 1)}


def eval_tessellation_math(fn, items):
    """rive_cuda_eval_tessellation_math: the tessellation kernel's device
    function `fn` on an (n, k_in) float32 array; returns (n, k_out)."""
    k_in, k_out = TESS_MATH_LAYOUT[fn]
    x = np.ascontiguousarray(items, np.float32).reshape(-1, k_in)
    out = np.zeros((len(x), k_out), np.float32)
    rc = load().rive_cuda_eval_tessellation_math(fn, x.ctypes.data_as(ctypes.c_void_p),
                                                 out.ctypes.data_as(ctypes.c_void_p), len(x))
    if rc != OK:
        raise RiveCudaError(f"eval_tessellation_math({fn}): status {rc}")
    return out


class Graph:
    """A batch captured as a CUDA graph (rive_cuda_graph_*)."""

    def __init__(self, ctx, handle):
        self.ctx, self.h = ctx, handle

    def launch(self, stream=None):
        self.ctx.check(self.ctx.lib.rive_cuda_graph_launch(self.h, stream), "graph_launch")

    def check(self, stream=None):
        self.ctx.check(self.ctx.lib.rive_cuda_graph_check(self.h, stream), "graph_check")

    def stats(self):
        s = FlushStats()
        self.ctx.check(self.ctx.lib.rive_cuda_graph_stats(self.h, ctypes.byref(s)), "graph_stats")
        return {k: getattr(s, k) for k, _ in FlushStats._fields_}

    def close(self):
        if self.h:
            self.ctx.lib.rive_cuda_graph_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Context:
    """One rive_cuda_context (one GPU, one stream)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = ctypes.c_void_p()
        rc = self.lib.rive_cuda_context_create(device, ctypes.byref(h))
        if rc != OK:
            raise RiveCudaError(f"rive_cuda_context_create failed ({rc})")
        self.h = h
        self._targets = []
        self._capacity = {}
        self._textures = {}  # id(capture.Texture) -> (texture, handle)
        self._buffers = {}  # id(capture.RenderBuffer) -> (buffer, handle)

    def close(self):
        if self.h:
            for t in self._targets:
                self.lib.rive_cuda_render_target_destroy(self.h, t)
            self._targets = []
            for _, handle in self._textures.values():
                self.lib.rive_cuda_texture_destroy(self.h, handle)
            self._textures = {}
            for _, handle in self._buffers.values():
                self.lib.rive_cuda_render_buffer_destroy(self.h, handle)
            self._buffers = {}
            self.lib.rive_cuda_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def error(self):
        buf = ctypes.create_string_buffer(512)
        self.lib.rive_cuda_last_error(self.h, buf, 512)
        return buf.value.decode()

    def check(self, rc, what):
        if rc != OK:
            raise RiveCudaError(f"{what}: status {rc}: {self.error()}")

    # -- RenderContextImpl-shaped calls -------------------------------------
    def resize_buffer(self, kind: int, nbytes: int):
        self.check(self.lib.rive_cuda_resize_buffer(self.h, kind, nbytes), "resize_buffer")
        self._capacity[kind] = nbytes

    def upload(self, kind: int, data: bytes):
        """resize (grow x1.25) / map / write / unmap, as RenderContext does."""
        n = len(data)
        if n == 0:
            return
        if self._capacity.get(kind, 0) < n:
            self.resize_buffer(kind, n + n // 4)
        p = self.lib.rive_cuda_map_buffer(self.h, kind, n)
        if not p:
            raise RiveCudaError(f"map_buffer failed: {self.error()}")
        ctypes.memmove(p, data, n)
        self.check(self.lib.rive_cuda_unmap_buffer(self.h, kind, n), "unmap_buffer")

    def render_target(self, width: int, height: int):
        t = ctypes.c_void_p()
        self.check(self.lib.rive_cuda_render_target_create(self.h, width, height, ctypes.byref(t)),
                   "render_target_create")
        self._targets.append(t)
        return t

    def textures_for(self, flush):
        """Device textures (rive_cuda_texture handles) for the capture
        textures a flush's batches sample, created once per texture."""
        if not getattr(flush, "has_images", False):
            return None
        out = []
        for t in flush.textures:
            key = id(t)
            if key not in self._textures:
                h = ctypes.c_void_p()
                data = np.frombuffer(t.rgba, np.uint8)
                self.check(self.lib.rive_cuda_texture_create(
                    self.h, t.width, t.height, t.mip_levels,
                    data.ctypes.data_as(ctypes.c_void_p), ctypes.byref(h)), "texture_create")
                self._textures[key] = (t, h)
            out.append(self._textures[key][1].value)
        return out

    def buffers_for(self, flush):
        """Device render buffers (rive_cuda_render_buffer handles) for the
        capture render buffers a flush's image meshes draw, created and
        written once per buffer."""
        if not getattr(flush, "has_meshes", False):
            return None
        out = []
        for b in flush.render_buffers:
            key = id(b)
            if key not in self._buffers:
                h = ctypes.c_void_p()
                data = np.frombuffer(b.data, np.uint8)
                self.check(self.lib.rive_cuda_render_buffer_create(
                    self.h, b.type, max(len(b.data), 1), ctypes.byref(h)), "render_buffer_create")
                self._buffers[key] = (b, h)
                if len(b.data):
                    self.check(self.lib.rive_cuda_render_buffer_write(
                        self.h, h, 0, data.ctypes.data_as(ctypes.c_void_p), len(b.data)),
                        "render_buffer_write")
            out.append(self._buffers[key][1].value)
        return out

    def desc_for(self, flush):
        """make_desc with this context's textures and render buffers."""
        return make_desc(flush, self.textures_for(flush), self.buffers_for(flush))

    def set_bin_speculation(self, enabled: bool):
        """rive_cuda_set_bin_speculation: flushes on the context's stream size
        their bins from the largest total seen instead of waiting for the
        scan (checked, and re-run exactly when short, at the next call)."""
        self.check(self.lib.rive_cuda_set_bin_speculation(self.h, int(bool(enabled))),
                   "set_bin_speculation")

    def read_texture(self, handle, level, width, height):
        """Mip level `level` (width x height texels) of a device texture."""
        out = np.zeros((height, width, 4), np.uint8)
        self.check(self.lib.rive_cuda_texture_read(self.h, ctypes.c_void_p(handle), level,
                                                    out.ctypes.data_as(ctypes.c_void_p),
                                                    out.nbytes), "texture_read")
        return out

    def flush(self, flush, target, stream=None):
        d, keep = self.desc_for(flush)
        self.check(self.lib.rive_cuda_flush(self.h, ctypes.byref(d), target, stream), "flush")
        del keep

    def flush_device(self, flush, bufs: DeviceBuffers, target_ptr: int, stream=None):
        d, keep = self.desc_for(flush)
        self.check(self.lib.rive_cuda_flush_device(self.h, ctypes.byref(d), ctypes.byref(bufs),
                                                   ctypes.c_void_p(target_ptr), stream),
                   "flush_device")
        del keep

    def _batch_array(self, items):
        arr = (BatchFlush * max(len(items), 1))()
        keep = []
        for i, (flush, bufs, target_ptr) in enumerate(items):
            d, k = self.desc_for(flush)
            keep.append((d, k))
            arr[i].desc = ctypes.cast(ctypes.pointer(d), ctypes.c_void_p)
            arr[i].buffers = bufs
            arr[i].target_pixels_device = target_ptr
        return arr, keep

    def flush_batch(self, items, stream=None):
        """rive_cuda_flush_batch over [(capture.Flush, DeviceBuffers, target_ptr), ...]:
        independent flushes (distinct targets) in one sequence of launches."""
        arr, keep = self._batch_array(items)
        self.check(self.lib.rive_cuda_flush_batch(self.h, arr, len(items), stream), "flush_batch")
        del keep

    def graph(self, items, bin_capacity=0):
        """rive_cuda_graph_create: the batch captured as one CUDA graph."""
        arr, keep = self._batch_array(items)
        g = ctypes.c_void_p()
        self.check(self.lib.rive_cuda_graph_create(self.h, arr, len(items), bin_capacity,
                                                   ctypes.byref(g)), "graph_create")
        del keep
        return Graph(self, g)

    def sync(self, stream=None):
        self.check(self.lib.rive_cuda_sync(self.h, stream), "sync")

    def read_target(self, target, width, height, out=None):
        if out is None:
            out = np.empty((height, width, 4), np.uint8)
        self.check(self.lib.rive_cuda_render_target_read(
            self.h, target, out.ctypes.data_as(ctypes.c_void_p), None), "render_target_read")
        return out

    def read_target_async(self, target, out_ptr: int, stream=None):
        """Enqueues the read-back into host memory at out_ptr (page-locked for
        an asynchronous copy; valid until sync(stream))."""
        self.check(self.lib.rive_cuda_render_target_read_async(
            self.h, target, ctypes.c_void_p(out_ptr), stream), "render_target_read_async")

    def target_device_ptr(self, target):
        return self.lib.rive_cuda_render_target_device_ptr(target)

    def read_tess(self, height):
        out = np.empty((height * 2048, 4), np.uint32)
        self.check(self.lib.rive_cuda_read_tess_texture(
            self.h, out.ctypes.data_as(ctypes.c_void_p), out.nbytes), "read_tess_texture")
        return out

    def read_atlas(self, width, height):
        """The feather atlas of the last flush, as float32 (from fp16)."""
        out = np.zeros((height, width), np.uint16)
        self.check(self.lib.rive_cuda_read_atlas_texture(
            self.h, out.ctypes.data_as(ctypes.c_void_p), out.nbytes), "read_atlas_texture")
        return out.view(np.float16).astype(np.float32)

    def read_grad(self, height):
        out = np.empty((height, 512, 4), np.uint8)
        self.check(self.lib.rive_cuda_read_grad_texture(
            self.h, out.ctypes.data_as(ctypes.c_void_p), out.nbytes), "read_grad_texture")
        return out

    def stats(self):
        s = FlushStats()
        self.check(self.lib.rive_cuda_last_flush_stats(self.h, ctypes.byref(s)), "stats")
        return {k: getattr(s, k) for k, _ in FlushStats._fields_}

    def set_profiling(self, on: bool):
        self.check(self.lib.rive_cuda_set_profiling(self.h, 1 if on else 0), "set_profiling")

    def set_raster_config(self, tile_size: int = 16, ctas_per_sm: int = 0):
        """Tile size (8, 16, 32) and resident raster CTAs per SM (0: as many as
        fit) for later flushes; the image is the same within tolerance."""
        self.check(self.lib.rive_cuda_set_raster_config(self.h, int(tile_size), int(ctas_per_sm)),
                   "set_raster_config")

    def set_winding_tiles(self, on: bool):
        """Interior tiles of fills as one winding record per path (on by
        default) or as the plain midpoint fan; the image is the same."""
        self.check(self.lib.rive_cuda_set_winding_tiles(self.h, 1 if on else 0),
                   "set_winding_tiles")

    def set_raster_queue(self, on: bool):
        """The raster as a persistent work queue over heaviest-first tiles
        (16-pixel tiles), or one CTA per tile (default); same image."""
        self.check(self.lib.rive_cuda_set_raster_queue(self.h, 1 if on else 0),
                   "set_raster_queue")

    def raster_queue(self):
        v = ctypes.c_int()
        self.check(self.lib.rive_cuda_get_raster_queue(self.h, ctypes.byref(v)),
                   "get_raster_queue")
        return bool(v.value)

    def winding_tiles(self):
        v = ctypes.c_int()
        self.check(self.lib.rive_cuda_get_winding_tiles(self.h, ctypes.byref(v)),
                   "get_winding_tiles")
        return bool(v.value)

    def raster_config(self):
        t, c = ctypes.c_int(), ctypes.c_int()
        self.check(self.lib.rive_cuda_get_raster_config(self.h, ctypes.byref(t), ctypes.byref(c)),
                   "get_raster_config")
        return t.value, c.value

    def profile_collect(self):
        ms = (ctypes.c_double * len(STAGES))()
        n = (ctypes.c_uint64 * len(STAGES))()
        self.check(self.lib.rive_cuda_profile_collect(self.h, ms, n), "profile_collect")
        return {st: (ms[i], n[i]) for i, st in enumerate(STAGES)}

    # -- helpers --------------------------------------------------------------
    def upload_frame(self, cap):
        for name in BUFFER_NAMES:
            self.upload(BUFFER_KINDS[name], cap.buffers.get(name, b""))

    def render(self, cap, target=None, read=True):
        """Uploads a captured frame, runs all its logical flushes, reads back."""
        if target is None:
            target = self.render_target(cap.width, cap.height)
        self.upload_frame(cap)
        for f in cap.flushes:
            self.flush(f, target)
        self.sync()
        if read:
            return self.read_target(target, cap.width, cap.height)
        return target
