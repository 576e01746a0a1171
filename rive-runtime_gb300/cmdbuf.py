"""Reader of the reference's deferred 2D command buffer, turned into a scene.

rive-runtime records Renderer/Factory calls into a RenderCommandBuffer
(renderer/include/rive/renderer/cmd/render_command_buffer.hpp): a flat,
pointer-free byte stream of [u8 opcode][POD payload] commands
(cmd/render_commands.hpp) plus a blob arena for variable-length data (path
verbs and points, gradient stops, encoded images, buffer contents), so a frame
can cross threads or processes. Its own consumer is replayRenderCommands
(cmd/render_replay.hpp, renderer/src/deferred_cmd.cpp), which rebuilds live
resources by dense id and drives a Renderer.

`command_buffer_scene` walks one frame's stream the same way and snapshots
every drawPath/clipPath into a `scene.Scene`, the planner's input: resources
are created, mutated, versioned (a resource drawn and then mutated again in
the same frame gets a new version; draws name the version they saw) and
destroyed by generation exactly as the replay does. Draws the replay would
drop (unresolved ids, content between canvas brackets, which needs a host
canvas) are dropped, and image draws and draws with feathered paints, which
this path does not render, are left out (feathered ones are kept with
`keep_feathered`); all are counted in `CmdbufStats`.

The payload layouts are the C structs' natural layouts (little-endian,
explicit padding); `POD_FORMATS` lists them by opcode.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

from . import scene as S

# RenderCmd (cmd/render_commands.hpp), in enum order.
OPCODES = [
    "makePath", "makeEmptyPath", "makePaint", "makeLinearGradient", "makeRadialGradient",
    "decodeImage", "makeBuffer", "bufferData", "destroyResource", "pathRewind", "pathFillRule",
    "pathAddRawPath", "pathAddRenderPath", "paintStyle", "paintColor", "paintThickness",
    "paintJoin", "paintCap", "paintFeather", "paintBlendMode", "paintShader",
    "paintInvalidateStroke", "save", "restore", "transform", "drawPath", "clipPath", "drawImage",
    "drawImageMesh", "modulateOpacity", "canvasContentBegin", "canvasContentEnd",
    "resourceNewVersion",
]
OP = {name: i for i, name in enumerate(OPCODES)}

# Payload of each opcode, as struct formats of the PODs (x = padding).
POD_FORMATS = {
    "makePath": "<IIQQIIII",          # MakePathPOD
    "makeEmptyPath": "<II",           # MakeIdPOD
    "makePaint": "<II",               # MakeIdPOD
    "makeLinearGradient": "<II4fQQII",  # LinearGradientPOD
    "makeRadialGradient": "<II3fIQQ",   # RadialGradientPOD
    "decodeImage": "<IIQIIII",        # DecodeImagePOD
    "makeBuffer": "<IIBBxxI",         # MakeBufferPOD
    "bufferData": "<QII",             # BufferDataPOD
    "destroyResource": "<BxxxII",     # DestroyResourcePOD
    "pathRewind": "<I",               # ResIdPOD
    "pathFillRule": "<IBxxx",         # PathFillRulePOD
    "pathAddRawPath": "<QQIIII",      # PathRawPOD
    "pathAddRenderPath": "<II6f",     # PathAddPathPOD
    "paintStyle": "<IBxxx",           # PaintU8POD
    "paintColor": "<II",              # PaintColorPOD
    "paintThickness": "<If",          # PaintFloatPOD
    "paintJoin": "<IBxxx",
    "paintCap": "<IBxxx",
    "paintFeather": "<If",
    "paintBlendMode": "<IBxxx",
    "paintShader": "<II",             # PaintShaderPOD
    "paintInvalidateStroke": "<I",
    "save": "",
    "restore": "",
    "transform": "<6f",               # TransformPOD
    "drawPath": "<IIII",              # DrawPathPOD
    "clipPath": "<II",                # ClipPathPOD
    "drawImage": "<IBBBBf",           # DrawImagePOD
    "drawImageMesh": "<9IBBBBf",      # DrawImageMeshPOD
    "modulateOpacity": "<f",          # OpacityPOD
    "canvasContentBegin": "<II",      # CanvasContentPOD
    "canvasContentEnd": "<I",
    "resourceNewVersion": "<BxxxII",  # ResourceVersionPOD
}
_STRUCTS = [struct.Struct(POD_FORMATS[n]) if POD_FORMATS[n] else None for n in OPCODES]

INVALID_HANDLE = 0xFFFFFFFF
# ResourceKind
KIND_PATH, KIND_PAINT, KIND_SHADER, KIND_IMAGE, KIND_BUFFER = range(5)

RCB_MAGIC = 0x31424352  # "RCB1": one self-contained frame
_RCB_HEADER = struct.Struct("<6IQQ")
RCS_MAGIC = 0x31534352  # "RCS1": a session, frame after frame
_RCS_HEADER = struct.Struct("<8I")
_RCS_FRAME = struct.Struct("<QQ")

_VERB_POINTS = {S.VERB_MOVE: 1, S.VERB_LINE: 1, S.VERB_QUAD: 2, S.VERB_CUBIC: 3,
                S.VERB_CLOSE: 0}


class CmdbufError(ValueError):
    pass


@dataclass
class CmdbufStats:
    draws: int = 0
    clips: int = 0
    dropped_unresolved: int = 0
    dropped_canvas: int = 0
    dropped_images: int = 0
    dropped_feathered: int = 0


def _map_points(m, pts):
    """Mat2D::mapPoints (src/math/mat2d.cpp:59-101) in float32."""
    m = np.asarray(m, np.float32)
    x, y = pts[:, 0], pts[:, 1]
    if m[1] == 0 and m[2] == 0:
        return np.stack([m[0] * x + m[4], m[3] * y + m[5]], 1).astype(np.float32)
    sx = m[2] * y + m[4]
    sy = m[1] * x + m[5]
    return np.stack([m[0] * x + sx, m[3] * y + sy], 1).astype(np.float32)


def _prune_empty_segments(verbs, pts, vstart=0, pstart=0):
    """RawPath::pruneEmptySegments(start) (src/math/raw_path.cpp:353-413):
    drops the lines, quads and cubics from verb `vstart` (point `pstart`) on
    whose points all equal the point before them."""
    out_v, out_p = list(verbs[:vstart]), [tuple(q) for q in pts[:pstart]]
    p = pstart
    for v in verbs[vstart:]:
        n = _VERB_POINTS[v]
        seg = [tuple(q) for q in pts[p:p + n]]
        empty = False
        if v in (S.VERB_LINE, S.VERB_QUAD, S.VERB_CUBIC) and p > 0:
            prev = tuple(pts[p - 1])
            chk = []
            if v == S.VERB_CUBIC:
                chk.append((seg[2], seg[1]))
            if v in (S.VERB_CUBIC, S.VERB_QUAD):
                chk.append((seg[1], seg[0]))
            chk.append((seg[0], prev))
            empty = all(a[0] == b[0] and a[1] == b[1] for a, b in chk)
        if not empty:
            out_v.append(v)
            out_p.extend(seg)
        p += n
    return out_v, (np.array(out_p, np.float32).reshape(-1, 2) if out_p
                   else np.zeros((0, 2), np.float32))


@dataclass
class _Path:
    verbs: list = field(default_factory=list)
    pts: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.float32))
    fill_rule: int = S.FILL_NONZERO
    serial: int = 0    # identity of the live object
    mutation: int = 0  # changes with every mutation


@dataclass
class _Paint:
    style: int = 1  # RenderPaintStyle::fill
    color: int = 0xFF000000
    thickness: float = 1.0
    join: int = 0
    cap: int = 0
    feather: float = 0.0
    blend_mode: int = 3
    shader: object = None  # the gradient the live paint holds
    serial: int = 0
    mutation: int = 0


class _Resident:
    """One resource type: dense ids, generations, versions and the per-frame
    aliases of outgoing versions (render_replay.hpp, Resident<T>)."""

    def __init__(self):
        self.objects, self.generations, self.versions = [], [], []
        self.aliases = {}

    def set(self, rid, obj, generation):
        if rid > len(self.objects):
            raise CmdbufError(f"resource id {rid} skips ahead of {len(self.objects)}")
        if rid == len(self.objects):
            self.objects.append(obj)
            self.generations.append(generation)
            self.versions.append(0)
            return
        self._drop_aliases(rid)
        self.objects[rid] = obj
        self.generations[rid] = generation
        self.versions[rid] = 0

    def _drop_aliases(self, rid):
        for k in [k for k in self.aliases if k[0] == rid]:
            del self.aliases[k]

    def new_version(self, rid, version, obj):
        if rid >= len(self.objects):
            return
        self.aliases[(rid, self.versions[rid])] = self.objects[rid]
        self.objects[rid] = obj
        self.versions[rid] = version

    def destroy(self, rid, generation):
        if rid < len(self.objects) and self.generations[rid] == generation:
            self.objects[rid] = None
            self._drop_aliases(rid)

    def get(self, rid, version=None):
        if rid >= len(self.objects):
            return None
        if version is None or version == self.versions[rid]:
            return self.objects[rid]
        return self.aliases.get((rid, version))


class CommandStreamReader:
    """Consumer side of a session's command stream, frame after frame: the
    resource tables persist across frames as they do on the reference's render
    thread (ResourceTable), and the aliases of outgoing versions live within
    one frame."""

    def __init__(self):
        self.paths, self.paints, self.shaders = _Resident(), _Resident(), _Resident()
        self.fill_rules, self.shadows = {}, {}
        self.serial = 0

    def skip_frame(self, commands: bytes, blobs: bytes):
        """Applies a frame's creates, mutations, versions and destroys without
        drawing it (a frame that is not shown)."""
        self._walk(commands, blobs, None, None)

    def frame_scene(self, commands: bytes, blobs: bytes, width: int, height: int,
                    clear_color: int = 0, dither_mode: int = S.DITHER_IGN, flags: int = 0,
                    keep_feathered: bool = False):
        """One frame's stream as (scene.Scene, CmdbufStats)."""
        sc = S.Scene(width, height, clear_color=clear_color, dither_mode=dither_mode,
                     flags=flags)
        st = CmdbufStats()
        self.keep_feathered = keep_feathered
        self._walk(commands, blobs, sc, st)
        return sc, st

    def _new_serial(self):
        self.serial += 1
        return self.serial

    def _walk(self, commands, blobs, sc, st):
        paths, paints, shaders = self.paths, self.paints, self.shaders
        fill_rules, shadows = self.fill_rules, self.shadows
        for r in (paths, paints, shaders):
            r.aliases.clear()
        draw = sc is not None
        new_serial = self._new_serial
        cmd = memoryview(commands)
        blob = memoryview(blobs)
        path_ix, paint_ix = {}, {}

        def blob_at(off, size):
            if off + size > len(blob):
                return None
            return bytes(blob[off:off + size])

        def raw_path(vo, po, nv, npts):
            vb = blob_at(vo, nv)
            pb = blob_at(po, 8 * npts)
            if vb is None or pb is None:
                return [], np.zeros((0, 2), np.float32)
            verbs = list(vb)
            need = 0
            for v in verbs:
                if v not in _VERB_POINTS:
                    raise CmdbufError(f"bad path verb {v}")
                need += _VERB_POINTS[v]
            if need != npts:
                raise CmdbufError(f"path verbs need {need} points, the stream has {npts}")
            pts = np.frombuffer(pb, "<f4").reshape(-1, 2).astype(np.float32)
            return verbs, pts

        def scene_path(p: _Path):
            key = (p.serial, p.mutation)
            if key not in path_ix:
                path_ix[key] = sc.add_path(S.Path(list(p.verbs), p.pts.copy(), p.fill_rule,
                                                  appended=True))
            return path_ix[key]

        def scene_paint(q: _Paint):
            key = (q.serial, q.mutation)
            if key not in paint_ix:
                p = S.Paint(style=S.STYLE_FILL if q.style == 1 else S.STYLE_STROKE, color=q.color,
                            thickness=q.thickness, join=q.join, cap=q.cap, blend_mode=q.blend_mode,
                            feather=q.feather)
                if q.shader is not None:
                    kind, stops, g = q.shader
                    p.shader, p.stops, p.g = kind, list(stops), tuple(g)
                paint_ix[key] = sc.add_paint(p)
            return paint_ix[key]

        def mutate(obj):
            obj.mutation += 1

        live = True  # False between canvas brackets: the replay drops those draws
        pos = 0
        n = len(cmd)
        while pos < n:
            op = cmd[pos]
            pos += 1
            if op >= len(OPCODES):
                raise CmdbufError(f"unknown opcode {op} at byte {pos - 1}")
            s = _STRUCTS[op]
            if s is not None:
                if pos + s.size > n:
                    raise CmdbufError("payload overrun")
                a = s.unpack_from(cmd, pos)
                pos += s.size
            else:
                a = ()
            name = OPCODES[op]
            if name == "makePath":
                rid, gen, vo, po, nv, npts, fr, _ = a
                verbs, pts = raw_path(vo, po, nv, npts)
                verbs, pts = _prune_empty_segments(verbs, pts)  # makeRenderPath prunes
                paths.set(rid, _Path(verbs, pts, fr, new_serial()), gen)
                fill_rules[rid] = fr
            elif name == "makeEmptyPath":
                rid, gen = a
                paths.set(rid, _Path(serial=new_serial()), gen)
                fill_rules[rid] = 0
            elif name == "makePaint":
                rid, gen = a
                paints.set(rid, _Paint(serial=new_serial()), gen)
                shadows[rid] = _Paint()
                shadows[rid].shader = INVALID_HANDLE
            elif name in ("makeLinearGradient", "makeRadialGradient"):
                if name == "makeLinearGradient":
                    rid, gen, sx, sy, ex, ey, co, so, count, _ = a
                    g = (sx, sy, ex, ey)
                    kind = S.SHADER_LINEAR
                else:
                    rid, gen, cx, cy, r, count, co, so = a
                    g = (cx, cy, r, 0.0)
                    kind = S.SHADER_RADIAL
                cb, sb = blob_at(co, 4 * count), blob_at(so, 4 * count)
                if cb is None or sb is None:
                    continue  # blob out of range: the replay skips it
                colors = struct.unpack(f"<{count}I", cb)
                stops = struct.unpack(f"<{count}f", sb)
                shaders.set(rid, (kind, list(zip(stops, colors)), g), gen)
            elif name == "decodeImage":
                pass  # images are not rendered on this path
            elif name in ("makeBuffer", "bufferData"):
                pass  # vertex/index buffers feed image meshes only
            elif name == "destroyResource":
                kind, rid, gen = a
                {KIND_PATH: paths, KIND_PAINT: paints, KIND_SHADER: shaders}.get(
                    kind, _Resident()).destroy(rid, gen)
            elif name == "resourceNewVersion":
                kind, rid, version = a
                if kind == KIND_PAINT:
                    sh = shadows.get(rid)
                    fresh = _Paint(serial=new_serial())
                    if sh is not None:
                        fresh.style, fresh.color, fresh.thickness = sh.style, sh.color, sh.thickness
                        fresh.join, fresh.cap, fresh.feather = sh.join, sh.cap, sh.feather
                        fresh.blend_mode = sh.blend_mode
                        if sh.shader != INVALID_HANDLE:
                            fresh.shader = shaders.get(sh.shader)
                    paints.new_version(rid, version, fresh)
                elif kind == KIND_PATH:
                    # Seeded from the outgoing version (addRenderPath with the
                    # identity matrix, which copies the raw path as is).
                    out = paths.get(rid)
                    fresh = _Path(serial=new_serial())
                    if out is not None:
                        fresh.verbs, fresh.pts = list(out.verbs), out.pts.copy()
                    fresh.fill_rule = fill_rules.get(rid, 0)
                    paths.new_version(rid, version, fresh)
            elif name == "pathRewind":
                p = paths.get(a[0])
                if p is not None:
                    p.verbs, p.pts = [], np.zeros((0, 2), np.float32)
                    mutate(p)
            elif name == "pathFillRule":
                p = paths.get(a[0])
                if p is not None:
                    p.fill_rule = a[1]
                    fill_rules[a[0]] = a[1]
                    mutate(p)
            elif name == "pathAddRawPath":
                vo, po, rid, nv, npts, _ = a
                verbs, pts = raw_path(vo, po, nv, npts)
                p = paths.get(rid)
                if p is not None:
                    p.verbs = p.verbs + verbs
                    p.pts = np.concatenate([p.pts, pts])
                    mutate(p)
            elif name == "pathAddRenderPath":
                rid, src_id, *m = a
                p, src = paths.get(rid), paths.get(src_id)
                if p is not None and src is not None:
                    # RiveRenderPath::addRenderPath (rive_render_path.cpp:83-98):
                    # a transformed copy has its now-empty segments pruned.
                    identity = tuple(m) == (1.0, 0.0, 0.0, 1.0, 0.0, 0.0)
                    v0, p0 = len(p.verbs), len(p.pts)
                    verbs = p.verbs + list(src.verbs)
                    if identity:
                        pts = np.concatenate([p.pts, src.pts])
                    else:
                        pts = np.concatenate([p.pts, _map_points(m, src.pts)])
                        verbs, pts = _prune_empty_segments(verbs, pts, v0, p0)
                    p.verbs, p.pts = verbs, pts
                    mutate(p)
            elif name in ("paintStyle", "paintColor", "paintThickness", "paintJoin", "paintCap",
                          "paintFeather", "paintBlendMode", "paintShader"):
                rid, v = a
                q = paints.get(rid)
                if q is None:
                    continue
                sh = shadows[rid]
                if name == "paintStyle":
                    q.style = sh.style = v
                elif name == "paintColor":
                    q.color = sh.color = v
                elif name == "paintThickness":
                    q.thickness = sh.thickness = v
                elif name == "paintJoin":
                    q.join = sh.join = v
                elif name == "paintCap":
                    q.cap = sh.cap = v
                elif name == "paintFeather":
                    q.feather = sh.feather = v
                elif name == "paintBlendMode":
                    q.blend_mode = sh.blend_mode = v
                else:
                    q.shader = shaders.get(v) if v != INVALID_HANDLE else None
                    sh.shader = v
                mutate(q)
            elif name == "paintInvalidateStroke":
                pass
            elif name in ("save", "restore"):
                if live and draw:
                    sc.cmd(S.CMD_SAVE if name == "save" else S.CMD_RESTORE)
            elif name == "transform":
                if live and draw:
                    sc.cmd(S.CMD_TRANSFORM, m=a)
            elif name == "modulateOpacity":
                if live and draw:
                    sc.cmd(S.CMD_MODULATE_OPACITY, m=(a[0], 0, 0, 0, 0, 0))
            elif name == "drawPath":
                pid, qid, pv, qv = a
                if not draw:
                    continue
                if not live:
                    st.dropped_canvas += 1
                    continue
                p, q = paths.get(pid, pv), paints.get(qid, qv)
                if p is None or q is None:
                    st.dropped_unresolved += 1
                    continue
                if q.feather != 0 and not getattr(self, "keep_feathered", False):
                    st.dropped_feathered += 1
                    continue
                st.draws += 1
                sc.cmd(S.CMD_DRAW_PATH, scene_path(p), scene_paint(q))
            elif name == "clipPath":
                pid, pv = a
                if not live or not draw:
                    continue
                p = paths.get(pid, pv)
                if p is not None:
                    st.clips += 1
                    sc.cmd(S.CMD_CLIP_PATH, scene_path(p))
            elif name in ("drawImage", "drawImageMesh"):
                if live and draw:
                    st.dropped_images += 1
            elif name == "canvasContentBegin":
                live = False
            elif name == "canvasContentEnd":
                live = True


def command_buffer_scene(commands: bytes, blobs: bytes, width: int, height: int,
                         clear_color: int = 0, dither_mode: int = S.DITHER_IGN,
                         flags: int = 0):
    """A self-contained frame stream (its resources created in the same
    stream) as (scene.Scene, CmdbufStats)."""
    return CommandStreamReader().frame_scene(commands, blobs, width, height, clear_color,
                                             dither_mode, flags)


def read_rcb(data: bytes):
    """A stored stream (.rcb: u32 magic 'RCB1', width, height, clear colour,
    dither mode, scene flags, u64 command bytes, u64 blob bytes, commands,
    blobs) as (commands, blobs, header dict)."""
    if len(data) < _RCB_HEADER.size:
        raise CmdbufError("truncated stream file")
    magic, w, h, clear, dither, flags, nc, nb = _RCB_HEADER.unpack_from(data, 0)
    if magic != RCB_MAGIC or _RCB_HEADER.size + nc + nb > len(data):
        raise CmdbufError("not a command-stream file")
    o = _RCB_HEADER.size
    return (bytes(data[o:o + nc]), bytes(data[o + nc:o + nc + nb]),
            dict(width=w, height=h, clear_color=clear, dither_mode=dither, flags=flags))


def rcb_scene(data: bytes, keep_feathered: bool = False):
    """A stored stream as (scene.Scene, CmdbufStats)."""
    commands, blobs, hdr = read_rcb(data)
    return CommandStreamReader().frame_scene(commands, blobs, keep_feathered=keep_feathered,
                                             **hdr)


def read_rcs(data: bytes):
    """A stored session (.rcs: u32 magic 'RCS1', width, height, clear colour,
    dither mode, scene flags, frame count, 0; then per frame u64 command
    bytes, u64 blob bytes, the commands, the blobs) as (frames
    [(commands, blobs)], header dict)."""
    if len(data) < _RCS_HEADER.size:
        raise CmdbufError("truncated session file")
    magic, w, h, clear, dither, flags, count, _ = _RCS_HEADER.unpack_from(data, 0)
    if magic != RCS_MAGIC:
        raise CmdbufError("not a command-session file")
    o = _RCS_HEADER.size
    frames = []
    for _ in range(count):
        if o + _RCS_FRAME.size > len(data):
            raise CmdbufError("truncated session file")
        nc, nb = _RCS_FRAME.unpack_from(data, o)
        o += _RCS_FRAME.size
        if o + nc + nb > len(data):
            raise CmdbufError("truncated session file")
        frames.append((bytes(data[o:o + nc]), bytes(data[o + nc:o + nc + nb])))
        o += nc + nb
    return frames, dict(width=w, height=h, clear_color=clear, dither_mode=dither, flags=flags)


def rcs_frame_scene(data: bytes, k: int):
    """Frame k of a stored session as (scene.Scene, CmdbufStats): frames
    0..k-1 are consumed for their resources, frame k is drawn."""
    frames, hdr = read_rcs(data)
    reader = CommandStreamReader()
    for commands, blobs in frames[:k]:
        reader.skip_frame(commands, blobs)
    return reader.frame_scene(*frames[k], **hdr)
