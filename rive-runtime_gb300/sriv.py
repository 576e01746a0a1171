"""Reader of .sriv renderer-call streams, turned into rive_scene frames.

A .sriv stream is what the reference's SerializingFactory records while an
artboard animates (utils/serializing_factory.cpp; wire opcodes in
include/utils/serialize_ops.hpp; the reference's own reader is
utils/serialized_replay.cpp). Layout: "SRIV", varuint version 1, then ops, each
a varuint opcode followed by its operands (varuints, little-endian float32s,
raw bytes). Factory ops create resources by id; RenderPath and RenderPaint
setters mutate them; Renderer ops draw; a `frame` op separates frames, so frame
0 is everything before the first `frame`.

`read_sriv` parses a stream; `SrivStream.frame_scene(k)` snapshots frame k as a
`scene.Scene`: every drawPath/clipPath records the path and paint as they are at
that call (one scene path/paint per distinct version), and save/restore,
transform and modulateOpacity carry over as commands. The renderer state is
per frame, as a test harness that calls Artboard::draw once per frame leaves
it (every draw is bracketed by save/restore).

Image draws and image meshes are dropped and counted in `FrameStats` unless
`images`: then each decodeImage's bytes are decoded (image_decode: PNG and
baseline JPEG) and premultiplied as RenderContext::decodeImage does
(render_context.cpp:237-262), drawImage becomes a scene image draw and
drawImageMesh a scene mesh of the RenderBuffer contents at that call, both
with ImageSampler::LinearClamp as the reference's replay draws them
(utils/serialized_replay.cpp:293-330). Draws with a feathered paint are
dropped and counted too unless `keep_feathered`.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

from . import scene as S

# SerializeOp (include/utils/serialize_ops.hpp).
OP_MAKE_RENDER_BUFFER = 0
OP_MAKE_LINEAR_GRADIENT = 1
OP_MAKE_RADIAL_GRADIENT = 2
OP_MAKE_RENDER_PATH = 3
OP_MAKE_RENDER_PAINT = 5
OP_DECODE_IMAGE = 6
OP_SAVE = 7
OP_RESTORE = 8
OP_TRANSFORM = 9
OP_DRAW_PATH = 10
OP_CLIP_PATH = 11
OP_DRAW_IMAGE = 12
OP_DRAW_IMAGE_MESH = 13
OP_SET_VERTEX_BUFFER_DATA = 14
OP_SET_INDEX_BUFFER_DATA = 15
OP_ADD_RAW_PATH = 16
OP_REWIND = 17
OP_FILL_RULE = 18
OP_STYLE = 20
OP_COLOR = 21
OP_THICKNESS = 22
OP_JOIN = 23
OP_CAP = 24
OP_FEATHER = 25
OP_BLEND_MODE = 26
OP_SHADER = 27
OP_FRAME = 28
OP_FRAME_SIZE = 29
OP_MODULATE_OPACITY = 30

_VERB_POINTS = {S.VERB_MOVE: 1, S.VERB_LINE: 1, S.VERB_QUAD: 2, S.VERB_CUBIC: 3,
                S.VERB_CLOSE: 0}


class SrivError(ValueError):
    pass


class _Reader:
    def __init__(self, data: bytes):
        self.b = memoryview(data)
        self.p = 0

    def done(self):
        return self.p >= len(self.b)

    def varuint(self) -> int:
        r = s = 0
        while True:
            if self.p >= len(self.b):
                raise SrivError("truncated varuint")
            c = self.b[self.p]
            self.p += 1
            r |= (c & 0x7F) << s
            s += 7
            if not c & 0x80:
                return r
            if s > 63:
                raise SrivError("varuint too long")

    def f32(self) -> float:
        if self.p + 4 > len(self.b):
            raise SrivError("truncated float")
        v = struct.unpack_from("<f", self.b, self.p)[0]
        self.p += 4
        return v

    def f32s(self, n) -> np.ndarray:
        if self.p + 4 * n > len(self.b):
            raise SrivError("truncated floats")
        v = np.frombuffer(self.b, dtype="<f4", count=n, offset=self.p).astype(np.float32)
        self.p += 4 * n
        return v

    def skip(self, n):
        if self.p + n > len(self.b):
            raise SrivError("truncated bytes")
        self.p += n


@dataclass
class _PathState:
    verbs: list = field(default_factory=list)
    points: list = field(default_factory=list)  # float32 (n, 2) chunks
    fill_rule: int = S.FILL_NONZERO
    version: int = 0


@dataclass
class _PaintState:
    # RenderPaint defaults (serializing_factory.cpp, SerializingRenderPaint).
    stroked: bool = False
    color: int = 0xFF000000
    thickness: float = 1.0
    join: int = S.JOIN_MITER
    cap: int = S.CAP_BUTT
    feather: float = 0.0
    blend_mode: int = S.BLEND_SRC_OVER
    shader: int | None = None
    version: int = 0


@dataclass
class FrameStats:
    draws: int = 0
    clips: int = 0
    dropped_feathered: int = 0
    dropped_images: int = 0
    images: int = 0
    meshes: int = 0


@dataclass
class _Call:
    op: int
    a: object = None
    b: object = None


@dataclass
class SrivStream:
    width: int
    height: int
    frames: list  # list of lists of _Call
    shaders: dict  # id -> (kind, stops [(pos, color)], g4)
    encoded_images: dict = field(default_factory=dict)  # id -> encoded bytes
    _decoded: dict = field(default_factory=dict)  # id -> premultiplied RGBA or None

    def decoded_image(self, iid):
        """The premultiplied RGBA8 texels of image `iid`, or None when it
        cannot be decoded here."""
        if iid not in self._decoded:
            from . import image_decode
            data = self.encoded_images.get(iid)
            try:
                self._decoded[iid] = (image_decode.premultiply(image_decode.decode(data))
                                      if data is not None else None)
            except image_decode.DecodeError:
                self._decoded[iid] = None
        return self._decoded[iid]

    def frame_scene(self, k: int, clear_color: int = 0x00000000,
                    dither_mode: int = S.DITHER_IGN, keep_feathered: bool = False,
                    images: bool = False):
        """Frame k as a scene.Scene plus its FrameStats."""
        sc = S.Scene(self.width, self.height, clear_color=clear_color, dither_mode=dither_mode)
        st = FrameStats()
        path_ix, paint_ix, image_ix, mesh_ix = {}, {}, {}, {}

        def image_of(iid):
            if iid not in image_ix:
                rgba = self.decoded_image(iid)
                image_ix[iid] = None if rgba is None else sc.add_image(S.Image(rgba))
            return image_ix[iid]

        def mesh_of(bufs):
            key = tuple((b[0], b[1]) for b in bufs)
            if key not in mesh_ix:
                pos, uv, idx = (b[3] for b in bufs)
                xy = np.frombuffer(pos, "<f4").reshape(-1, 2)
                tc = np.zeros_like(xy)
                uvs = np.frombuffer(uv, "<f4")[:2 * len(xy)].reshape(-1, 2)
                tc[:len(uvs)] = uvs
                ix = np.frombuffer(idx, "<u2")
                ix = ix[:len(ix) - len(ix) % 3]
                mesh_ix[key] = sc.add_mesh(S.Mesh(xy, tc, ix)) if len(ix) and len(xy) else None
            return mesh_ix[key]

        def path_of(snap):
            key = snap[0]
            if key not in path_ix:
                _, verbs, pts, fill_rule = snap
                # The reference's replay builds every path with
                # makeEmptyRenderPath + addRawPath.
                path_ix[key] = sc.add_path(S.Path(verbs, pts, fill_rule, appended=True))
            return path_ix[key]

        def paint_of(snap):
            key = snap[0]
            if key not in paint_ix:
                q = snap[1]
                p = S.Paint(style=S.STYLE_STROKE if q.stroked else S.STYLE_FILL,
                            color=q.color, thickness=q.thickness, join=q.join, cap=q.cap,
                            blend_mode=q.blend_mode, feather=q.feather)
                sh = self.shaders.get(q.shader) if q.shader is not None else None
                if sh is not None:
                    kind, stops, g = sh
                    p.shader, p.stops, p.g = kind, list(stops), tuple(g)
                paint_ix[key] = sc.add_paint(p)
            return paint_ix[key]

        for c in self.frames[k]:
            if c.op == OP_SAVE:
                sc.cmd(S.CMD_SAVE)
            elif c.op == OP_RESTORE:
                sc.cmd(S.CMD_RESTORE)
            elif c.op == OP_TRANSFORM:
                sc.cmd(S.CMD_TRANSFORM, m=c.a)
            elif c.op == OP_MODULATE_OPACITY:
                sc.cmd(S.CMD_MODULATE_OPACITY, m=(c.a, 0, 0, 0, 0, 0))
            elif c.op == OP_CLIP_PATH:
                st.clips += 1
                sc.cmd(S.CMD_CLIP_PATH, path_of(c.a))
            elif c.op == OP_DRAW_PATH:
                if c.b[1].feather != 0 and not keep_feathered:
                    st.dropped_feathered += 1
                    continue
                st.draws += 1
                sc.cmd(S.CMD_DRAW_PATH, path_of(c.a), paint_of(c.b))
            elif c.op in (OP_DRAW_IMAGE, OP_DRAW_IMAGE_MESH):
                im = image_of(c.a[0]) if images else None
                if im is None:
                    st.dropped_images += 1
                    continue
                iid, blend, opacity = c.a
                if c.op == OP_DRAW_IMAGE:
                    st.images += 1
                    sc.draw_image(im, opacity, blend, S.sampler_key())
                else:
                    mi = mesh_of(c.b)
                    if mi is None:
                        st.dropped_images += 1
                        continue
                    st.meshes += 1
                    sc.draw_image_mesh(im, mi, opacity, blend, S.sampler_key())
        return sc, st


FRAMES_MAGIC = b"RSA1"


def pack_frames(frames) -> bytes:
    """A sequence of scene recordings (rive_scene.h bytes, one per frame) in
    one compressed container: "RSA1", u32 count, u32 offsets[count + 1] into
    the zlib-compressed concatenation that follows."""
    import zlib
    offs = [0]
    for f in frames:
        offs.append(offs[-1] + len(f))
    head = FRAMES_MAGIC + struct.pack(f"<{len(offs) + 1}I", len(frames), *offs)
    return head + zlib.compress(b"".join(frames), 9)


def unpack_frames(data: bytes) -> list:
    """The scene recordings of a pack_frames container."""
    import zlib
    if data[:4] != FRAMES_MAGIC:
        raise SrivError("not a frame container")
    (n,) = struct.unpack_from("<I", data, 4)
    offs = struct.unpack_from(f"<{n + 1}I", data, 8)
    body = zlib.decompress(data[8 + 4 * (n + 1):])
    if len(body) != offs[-1]:
        raise SrivError("frame container size mismatch")
    return [body[offs[i]:offs[i + 1]] for i in range(n)]


def read_sriv(data: bytes, default_size=None) -> SrivStream:
    """Parses a whole .sriv stream (utils/serialized_replay.cpp reads the same
    layout); raises SrivError on a malformed or truncated stream. A stream
    without a frameSize op takes `default_size` (width, height), else fails."""
    r = _Reader(data)
    if bytes(r.b[:4]) != b"SRIV":
        raise SrivError("not a .sriv stream")
    r.skip(4)
    if r.varuint() != 1:
        raise SrivError("unsupported .sriv version")
    paths: dict[int, _PathState] = {}
    paints: dict[int, _PaintState] = {}
    shaders: dict[int, tuple] = {}
    buffers: dict[int, list] = {}  # id -> [size, type, version, bytes]
    encoded: dict[int, bytes] = {}
    frames = [[]]
    width = height = 0
    serial = [0]

    def bump(state):
        serial[0] += 1
        state.version = serial[0]

    def path_snap(pid):
        p = paths.get(pid)
        if p is None:
            raise SrivError(f"unknown path {pid}")
        pts = (np.concatenate(p.points) if p.points else np.zeros((0, 2), np.float32))
        return (("path", pid, p.version), list(p.verbs), pts, p.fill_rule)

    def paint_snap(qid):
        q = paints.get(qid)
        if q is None:
            raise SrivError(f"unknown paint {qid}")
        return (("paint", qid, q.version), _PaintState(**q.__dict__))

    def paint(qid):
        q = paints.get(qid)
        if q is None:
            raise SrivError(f"unknown paint {qid}")
        return q

    while not r.done():
        op = r.varuint()
        if op == OP_MAKE_RENDER_PATH:
            pid = r.varuint()
            paths[pid] = _PathState()
            bump(paths[pid])
        elif op == OP_MAKE_RENDER_PAINT:
            qid = r.varuint()
            paints[qid] = _PaintState()
            bump(paints[qid])
        elif op == OP_REWIND:
            pid = r.varuint()
            if pid not in paths:
                raise SrivError(f"unknown path {pid}")
            p = paths[pid]
            p.verbs, p.points = [], []
            bump(p)
        elif op == OP_FILL_RULE:
            pid = r.varuint()
            rule = r.varuint()
            if pid not in paths:
                raise SrivError(f"unknown path {pid}")
            if rule > S.FILL_CLOCKWISE:
                raise SrivError(f"bad fill rule {rule}")
            paths[pid].fill_rule = rule
            bump(paths[pid])
        elif op == OP_ADD_RAW_PATH:
            pid = r.varuint()
            if pid not in paths:
                raise SrivError(f"unknown path {pid}")
            nv = r.varuint()
            verbs = [r.varuint() for _ in range(nv)]
            npts = r.varuint()
            pts = r.f32s(2 * npts).reshape(-1, 2)
            # deserializeRawPath stops at the first verb whose points are
            # missing; keep the verbs that have them.
            need, kept = 0, []
            for v in verbs:
                if v not in _VERB_POINTS:
                    raise SrivError(f"bad verb {v}")
                if need + _VERB_POINTS[v] > npts:
                    break
                need += _VERB_POINTS[v]
                kept.append(v)
            p = paths[pid]
            p.verbs.extend(kept)
            p.points.append(pts[:need])
            bump(p)
        elif op in (OP_COLOR, OP_STYLE, OP_JOIN, OP_CAP, OP_BLEND_MODE):
            q = paint(r.varuint())
            v = r.varuint()
            if op in (OP_JOIN, OP_CAP) and v > 2 or op == OP_BLEND_MODE and v > 28:
                raise SrivError(f"bad paint value {v} for opcode {op}")
            if op == OP_COLOR:
                q.color = v & 0xFFFFFFFF
            elif op == OP_STYLE:
                q.stroked = v == 0  # the stream writes 0 for stroke, 1 for fill
            elif op == OP_JOIN:
                q.join = v
            elif op == OP_CAP:
                q.cap = v
            else:
                q.blend_mode = v
            bump(q)
        elif op in (OP_THICKNESS, OP_FEATHER):
            q = paint(r.varuint())
            v = r.f32()
            if op == OP_THICKNESS:
                q.thickness = v
            else:
                q.feather = v
            bump(q)
        elif op == OP_SHADER:
            q = paint(r.varuint())
            sid = r.varuint()
            # 0 stands for both "no shader" and shader id 0; as in the
            # reference's replay, an id with no gradient means none.
            q.shader = sid if sid in shaders else None
            bump(q)
        elif op in (OP_MAKE_LINEAR_GRADIENT, OP_MAKE_RADIAL_GRADIENT):
            sid = r.varuint()
            n = r.varuint()
            stops = []
            for _ in range(n):
                color = r.varuint() & 0xFFFFFFFF
                stops.append((r.f32(), color))
            if op == OP_MAKE_LINEAR_GRADIENT:
                g = (r.f32(), r.f32(), r.f32(), r.f32())
                shaders[sid] = (S.SHADER_LINEAR, stops, g)
            else:
                g = (r.f32(), r.f32(), r.f32(), 0.0)
                shaders[sid] = (S.SHADER_RADIAL, stops, g)
        elif op == OP_DECODE_IMAGE:
            iid = r.varuint()
            n = r.varuint()
            start = r.p
            r.skip(n)
            encoded[iid] = bytes(r.b[start:start + n])
        elif op == OP_MAKE_RENDER_BUFFER:
            bid = r.varuint()
            size = r.varuint()
            kind = r.varuint()  # RenderBufferType
            r.varuint()  # RenderBufferFlags
            buffers[bid] = [size, kind, 0, bytes(size)]
        elif op in (OP_SET_VERTEX_BUFFER_DATA, OP_SET_INDEX_BUFFER_DATA):
            bid = r.varuint()
            if bid not in buffers:
                raise SrivError(f"unknown buffer {bid}")
            size = buffers[bid][0]
            if op == OP_SET_VERTEX_BUFFER_DATA:
                data_bytes = bytes(r.f32s(size // 4).astype("<f4").tobytes())
            else:
                vals = [r.varuint() & 0xFFFF for _ in range(size // 2)]
                data_bytes = np.array(vals, "<u2").tobytes()
            buf = buffers[bid]
            buf[3] = data_bytes + bytes(size - len(data_bytes))
            serial[0] += 1
            buf[2] = serial[0]
        elif op == OP_SAVE or op == OP_RESTORE:
            frames[-1].append(_Call(op))
        elif op == OP_TRANSFORM:
            frames[-1].append(_Call(op, tuple(float(v) for v in r.f32s(6))))
        elif op == OP_MODULATE_OPACITY:
            frames[-1].append(_Call(op, r.f32()))
        elif op == OP_DRAW_PATH:
            pid = r.varuint()
            qid = r.varuint()
            frames[-1].append(_Call(op, path_snap(pid), paint_snap(qid)))
        elif op == OP_CLIP_PATH:
            frames[-1].append(_Call(op, path_snap(r.varuint())))
        elif op == OP_DRAW_IMAGE:
            iid = r.varuint()
            blend = r.varuint()
            opacity = float(r.f32())
            frames[-1].append(_Call(op, (iid, blend, opacity)))
        elif op == OP_DRAW_IMAGE_MESH:
            iid = r.varuint()
            blend = r.varuint()
            opacity = float(r.f32())
            ids = [r.varuint() for _ in range(3)]
            # The buffers' contents at this call: (id, version, type, bytes).
            snaps = tuple((b, buffers[b][2], buffers[b][1], buffers[b][3]) if b in buffers
                          else (b, -1, 0, b"") for b in ids)
            frames[-1].append(_Call(op, (iid, blend, opacity), snaps))
        elif op == OP_FRAME:
            frames.append([])
        elif op == OP_FRAME_SIZE:
            width, height = r.varuint(), r.varuint()
        else:
            raise SrivError(f"unknown opcode {op}")
    if (width == 0 or height == 0) and default_size:
        width, height = default_size
    if width == 0 or height == 0:
        raise SrivError("no frame size")
    return SrivStream(width, height, frames, shaders, encoded)
