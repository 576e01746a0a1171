"""Reader/writer for flush captures: the frame's record buffers plus the list
of logical flushes (rive_cuda_flush_desc + rive_cuda_draw_batch[]).

A capture is exactly what rive::gpu::RenderContext hands its RenderContextImpl
for one frame (render_context.cpp:970-1010): the bytes written into the mapped
path/paint/paintAux/contour/gradSpan/tessVertexSpan/flushUniform buffers, and
one gpu::FlushDescriptor per logical flush. A frame that renders into the
feather atlas or draws images is an "RCP2" capture: each flush also carries
the atlas sizes, its gpu::AtlasDrawBatch lists (gpu.hpp:827-833, 1361-1426)
and each draw batch's image (texture index and ImageSampler key), and the
capture ends with the image textures the front end created
(RenderContextImpl::makeImageTexture: size, mip levels, level-0 RGBA).
A frame that draws image meshes is an "RCP3" capture: an RCP2 capture whose
flushes also name each imageMesh batch's vertex, uv and index RenderBuffers
and index count, whose buffers include the ImageDrawInstance records, and
which ends with the RenderBuffer contents each flush drew
(RenderContextImpl::makeRenderBuffer; a buffer rewritten between flushes
appears once per distinct content).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

CAPTURE_MAGIC = 0x31504352  # "RCP1"
CAPTURE_MAGIC_V2 = 0x32504352  # "RCP2": with feather atlas batches
CAPTURE_MAGIC_V3 = 0x33504352  # "RCP3": RCP2 with image meshes

BUFFER_NAMES = ("flush_uniforms", "paths", "paints", "paint_aux", "contours",
                "grad_spans", "tess_spans", "triangles", "image_draws")
NO_BUFFER = 0xFFFFFFFF

# rive_cuda_flush_desc field order (include/rive_cuda.h); 36 u32-sized fields,
# then the draw_batches pointer (8 bytes, LP64).
DESC_FIELDS = (
    "render_target_width", "render_target_height", "interlock_mode",
    "color_load_action", "color_clear_value", "ub0", "ub1", "ub2", "ub3",
    "combined_shader_features", "dither_mode", "flush_uniform_offset_bytes",
    "path_count", "first_path", "first_paint", "first_paint_aux",
    "contour_count", "first_contour", "grad_span_count", "first_grad_span",
    "tess_span_count", "first_tess_span", "grad_data_height",
    "tess_data_height", "grad_texture_height", "wireframe",
    "clockwise_fill_override", "has_triangle_vertices", "draw_batch_count",
)
DESC_STRUCT = struct.Struct("<5I4i20I")
DESC_SIZE = 128  # 29 fields * 4 = 116, pad 4, + 8-byte draw_batches pointer (LP64)
BATCH_FIELDS = ("draw_type", "element_count", "base_element", "shader_features",
                "draw_contents", "shader_misc_flags", "first_blend_mode",
                "barriers")
BATCH_SIZE = 32
# The atlas part of an RCP2 flush: these six u32 fields, then the atlas
# batches (fill batches first), 16 bytes each: u16 scissor left, top, right,
# bottom, u32 patch_count, u32 base_patch. Held per flush as an (n, 4) uint32
# array: [left | top << 16, right | bottom << 16, patch_count, base_patch].
ATLAS_FIELDS = ("atlas_texture_width", "atlas_texture_height", "atlas_content_width",
                "atlas_content_height", "atlas_fill_batch_count", "atlas_stroke_batch_count")


@dataclass
class Texture:
    width: int
    height: int
    mip_levels: int
    rgba: bytes  # level 0, premultiplied RGBA8, row 0 at the top


@dataclass
class RenderBuffer:
    type: int  # rive::RenderBufferType: 0 index, 1 vertex
    data: bytes


@dataclass
class Flush:
    desc: dict
    batches: np.ndarray  # (n, 8) uint32
    atlas: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.uint32))
    # Per draw batch: (texture index or 0xffffffff, sampler key); empty when
    # no batch draws an image.
    images: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.uint32))
    # The capture's textures (the indices above refer to them).
    textures: list = field(default_factory=list)
    # Per draw batch: (vertex buffer, uv buffer, index buffer, index count),
    # buffers as indices into render_buffers (NO_BUFFER: not a mesh); empty
    # when no batch draws an image mesh.
    meshes: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.uint32))
    render_buffers: list = field(default_factory=list)

    @property
    def has_atlas(self) -> bool:
        return any(self.desc.get(k, 0) for k in ATLAS_FIELDS)

    @property
    def has_images(self) -> bool:
        return bool(len(self.images)) and bool((self.images[:, 0] != 0xFFFFFFFF).any())

    @property
    def has_meshes(self) -> bool:
        return bool(len(self.meshes)) and bool((self.meshes[:, 0] != NO_BUFFER).any())


@dataclass
class Capture:
    width: int
    height: int
    buffers: dict = field(default_factory=dict)  # name -> bytes
    flushes: list = field(default_factory=list)
    textures: list = field(default_factory=list)  # Texture
    render_buffers: list = field(default_factory=list)  # RenderBuffer

    def buffer_array(self, name, dtype=np.uint32):
        return np.frombuffer(self.buffers[name], dtype=dtype)

    @property
    def tess_span_count(self):
        return len(self.buffers["tess_spans"]) // 64


def parse(data: bytes) -> Capture:
    magic, w, h, nk = struct.unpack_from("<4I", data, 0)
    if magic not in (CAPTURE_MAGIC, CAPTURE_MAGIC_V2, CAPTURE_MAGIC_V3):
        raise ValueError("not a flush capture")
    v3 = magic == CAPTURE_MAGIC_V3
    v2 = v3 or magic == CAPTURE_MAGIC_V2
    off = 16
    cap = Capture(w, h)
    for k in range(nk):
        (n,) = struct.unpack_from("<Q", data, off)
        off += 8
        cap.buffers[BUFFER_NAMES[k]] = bytes(data[off:off + n])
        off += n + ((8 - (n & 7)) & 7)
    (nf,) = struct.unpack_from("<I", data, off)
    off += 4
    for _ in range(nf):
        vals = DESC_STRUCT.unpack_from(data, off)
        desc = dict(zip(DESC_FIELDS, vals))
        off += DESC_SIZE
        nb = desc["draw_batch_count"]
        batches = np.frombuffer(data, dtype="<u4", count=nb * 8, offset=off).reshape(nb, 8).copy()
        off += nb * BATCH_SIZE
        atlas = np.zeros((0, 4), np.uint32)
        for k in ATLAS_FIELDS:
            desc[k] = 0
        if v2:
            vals = struct.unpack_from("<6I", data, off)
            off += 24
            desc.update(zip(ATLAS_FIELDS, vals))
            na = vals[4] + vals[5]
            atlas = np.frombuffer(data, dtype="<u4", count=na * 4, offset=off).reshape(na, 4).copy()
            off += na * 16
            (ni,) = struct.unpack_from("<I", data, off)
            off += 4
            images = np.frombuffer(data, dtype="<u4", count=ni * 2, offset=off).reshape(ni, 2).copy()
            off += ni * 8
        else:
            images = np.zeros((0, 2), np.uint32)
        meshes = np.zeros((0, 4), np.uint32)
        if v3:
            (nm,) = struct.unpack_from("<I", data, off)
            off += 4
            meshes = np.frombuffer(data, dtype="<u4", count=nm * 4, offset=off).reshape(nm, 4).copy()
            off += nm * 16
        cap.flushes.append(Flush(desc, batches, atlas, images, meshes=meshes))
    if v2:
        (nt,) = struct.unpack_from("<I", data, off)
        off += 4
        for _ in range(nt):
            w, h, levels = struct.unpack_from("<3I", data, off)
            off += 12
            cap.textures.append(Texture(w, h, levels, bytes(data[off:off + w * h * 4])))
            off += w * h * 4
    if v3:
        (nb,) = struct.unpack_from("<I", data, off)
        off += 4
        for _ in range(nb):
            kind, n = struct.unpack_from("<2I", data, off)
            off += 8
            cap.render_buffers.append(RenderBuffer(kind, bytes(data[off:off + n])))
            off += n + ((4 - (n & 3)) & 3)
    for f in cap.flushes:
        f.textures = cap.textures
        f.render_buffers = cap.render_buffers
    return cap


def serialize(cap: Capture) -> bytes:
    # Seven kinds, eight when the frame has interior triangles, nine when it
    # has image draw instances.
    kinds = BUFFER_NAMES if cap.buffers.get("image_draws") else \
        BUFFER_NAMES[:8] if cap.buffers.get("triangles") else BUFFER_NAMES[:7]
    v3 = any(f.has_meshes for f in cap.flushes) or bool(cap.render_buffers)
    v2 = v3 or any(f.has_atlas or f.has_images for f in cap.flushes) or bool(cap.textures)
    magic = CAPTURE_MAGIC_V3 if v3 else CAPTURE_MAGIC_V2 if v2 else CAPTURE_MAGIC
    out = bytearray(struct.pack("<4I", magic, cap.width, cap.height, len(kinds)))
    for name in kinds:
        b = cap.buffers.get(name, b"")
        out += struct.pack("<Q", len(b)) + b + bytes((8 - (len(b) & 7)) & 7)
    out += struct.pack("<I", len(cap.flushes))
    for f in cap.flushes:
        d = dict(f.desc)
        d["draw_batch_count"] = len(f.batches)
        out += DESC_STRUCT.pack(*[d[k] for k in DESC_FIELDS])
        out += bytes(DESC_SIZE - DESC_STRUCT.size)
        out += np.asarray(f.batches, dtype="<u4").tobytes()
        if v2:
            out += struct.pack("<6I", *[d.get(k, 0) for k in ATLAS_FIELDS])
            out += np.asarray(f.atlas, dtype="<u4").reshape(-1, 4).tobytes()
            im = np.asarray(f.images, dtype="<u4").reshape(-1, 2) if f.has_images else \
                np.zeros((0, 2), "<u4")
            out += struct.pack("<I", len(im)) + im.tobytes()
        if v3:
            me = np.asarray(f.meshes, dtype="<u4").reshape(-1, 4) if f.has_meshes else \
                np.zeros((0, 4), "<u4")
            out += struct.pack("<I", len(me)) + me.tobytes()
    if v2:
        out += struct.pack("<I", len(cap.textures))
        for t in cap.textures:
            out += struct.pack("<3I", t.width, t.height, t.mip_levels) + bytes(t.rgba)
    if v3:
        out += struct.pack("<I", len(cap.render_buffers))
        for b in cap.render_buffers:
            n = len(b.data)
            out += struct.pack("<2I", b.type, n) + bytes(b.data) + bytes((4 - (n & 3)) & 3)
    return bytes(out)
