"""Seeded synthetic scenes, written in the rive_scene.h recording format.

A scene is the list of rive::Renderer / rive::Factory calls that make one frame
(include/rive/renderer.hpp:212-236, include/rive/factory.hpp:35-87): paths
(RawPath + FillRule), paints (RiveRenderPaint, renderer/src/rive_render_paint.hpp)
and save/restore/transform/clipPath/drawPath commands.

The workloads:

* ``plain_small``: a 512x512 canvas cleared to opaque white; 200 closed filled
  paths, each one contour of 8 cubics with every control point uniform in
  [0,512)^2; nonzero; identity transforms; solid colours with RGB uniform in
  [0,1] and alpha uniform in [0.5,1]; srcOver; painter's order.
* ``full_feature``: a 2048x2048 canvas, 5,000 paths. 60% fills (half nonzero,
  half even-odd; 1-4 contours of 4-64 cubics), 40% strokes (width
  lognormal(ln 4, 0.7); joins miter/round/bevel; caps butt/round/square).
  Each path has an affine transform: rotation U[0, 2pi), scale log-U[0.25, 4],
  translation U(canvas). 30% of paints are linear/radial gradients with 2-8
  stops, 10% use a blend mode drawn from the 16 modes, 10% sit under nested
  clip paths of depth 1-3. Path geometry is drawn in a local box of
  [-LOCAL_HALF_EXTENT, LOCAL_HALF_EXTENT]^2 before its transform.
* ``stroke_stress``: strokes of 1-16 cubics, 20% of them cusps or
  near-degenerate; width log-U[0.5, 64]; round joins and caps; alpha 0.8.

Everything is drawn from numpy's PCG64 generator, so the same seed gives the
same bytes on every machine.
"""
from __future__ import annotations

import math
import struct
from dataclasses import dataclass, field

import numpy as np

MAGIC = 0x31435352  # "RSC1"

VERB_MOVE, VERB_LINE, VERB_QUAD, VERB_CUBIC, VERB_CLOSE = 0, 1, 2, 4, 5
CMD_SAVE, CMD_RESTORE, CMD_TRANSFORM, CMD_DRAW_PATH, CMD_CLIP_PATH = 0, 1, 2, 3, 4
CMD_MODULATE_OPACITY = 5  # m[0] = opacity (Renderer::modulateOpacity)
# Renderer::drawImage: a = image index, b = blend mode | sampler key << 8,
# m[0] = opacity.
CMD_DRAW_IMAGE = 6
IMAGES_MAGIC = 0x31495352  # "RSI1"
# Renderer::drawImageMesh: a = image index, b = blend mode | sampler key << 8,
# m[0] = opacity, m[1] = mesh index.
CMD_DRAW_IMAGE_MESH = 7
MESHES_MAGIC = 0x314D5352  # "RSM1"
# ImageSampler (include/rive/shapes/paint/image_sampler.hpp): key =
# wrapX + 3 wrapY + 9 filter; wrap 0 clamp, 1 repeat, 2 mirror; filter 0
# bilinear, 1 nearest.
WRAP_CLAMP, WRAP_REPEAT, WRAP_MIRROR = 0, 1, 2
FILTER_BILINEAR, FILTER_NEAREST = 0, 1


def sampler_key(wrap_x=WRAP_CLAMP, wrap_y=WRAP_CLAMP, filt=FILTER_BILINEAR) -> int:
    return wrap_x + 3 * wrap_y + 9 * filt
STYLE_STROKE, STYLE_FILL = 0, 1
SHADER_NONE, SHADER_LINEAR, SHADER_RADIAL = 0, 1, 2
FILL_NONZERO, FILL_EVENODD, FILL_CLOCKWISE = 0, 1, 2
PATH_APPENDED = 0x100  # rive_scene_path.fill_rule flag
JOIN_MITER, JOIN_ROUND, JOIN_BEVEL = 0, 1, 2
CAP_BUTT, CAP_ROUND, CAP_SQUARE = 0, 1, 2

# rive::BlendMode values (include/rive/shapes/paint/blend_mode.hpp).
BLEND_SRC_OVER = 3
BLEND_MODES = [3, 14, 15, 16, 17, 18, 19, 20, 21, 22, 23, 24, 25, 26, 27, 28]

LOCAL_HALF_EXTENT = 48.0

DITHER_NONE, DITHER_IGN = 0, 1
FLAG_TRIANGULATE = 1
FLAG_FEATHER_ATLAS = 2  # every feather through the feather atlas (alwaysFeatherToAtlas)


@dataclass
class Path:
    verbs: list
    points: np.ndarray  # float32 (n, 2)
    fill_rule: int = FILL_NONZERO
    # Built by makeEmptyRenderPath + addRawPath (a replayed call stream):
    # empty segments are kept instead of pruned.
    appended: bool = False


@dataclass
class Paint:
    style: int = STYLE_FILL
    color: int = 0xFF000000
    thickness: float = 1.0
    join: int = JOIN_MITER
    cap: int = CAP_BUTT
    blend_mode: int = BLEND_SRC_OVER
    shader: int = SHADER_NONE
    g: tuple = (0.0, 0.0, 0.0, 0.0)
    stops: list = field(default_factory=list)  # [(pos, color)]
    feather: float = 0.0  # RenderPaint::feather


@dataclass
class Image:
    """RGBA8 premultiplied texels, (height, width, 4) uint8, row 0 at the top."""
    rgba: np.ndarray


@dataclass
class Mesh:
    """An image mesh: local positions (n, 2), texture coordinates (n, 2) and a
    uint16 triangle list."""
    xy: np.ndarray
    uv: np.ndarray
    indices: np.ndarray


@dataclass
class Scene:
    width: int
    height: int
    clear_color: int = 0xFFFFFFFF
    dither_mode: int = DITHER_IGN
    flags: int = 0  # FLAG_TRIANGULATE: let the front end triangulate large fills
    paths: list = field(default_factory=list)
    paints: list = field(default_factory=list)
    cmds: list = field(default_factory=list)  # (op, a, b, m6)
    images: list = field(default_factory=list)  # Image
    meshes: list = field(default_factory=list)  # Mesh

    def add_path(self, p: Path) -> int:
        self.paths.append(p)
        return len(self.paths) - 1

    def add_paint(self, p: Paint) -> int:
        self.paints.append(p)
        return len(self.paints) - 1

    def add_image(self, im: Image) -> int:
        self.images.append(im)
        return len(self.images) - 1

    def draw_image(self, image: int, opacity: float = 1.0, blend_mode: int = BLEND_SRC_OVER,
                   sampler: int = 0):
        self.cmd(CMD_DRAW_IMAGE, image, blend_mode | (sampler << 8), (opacity, 0, 0, 0, 0, 0))

    def add_mesh(self, m: Mesh) -> int:
        self.meshes.append(m)
        return len(self.meshes) - 1

    def draw_image_mesh(self, image: int, mesh: int, opacity: float = 1.0,
                        blend_mode: int = BLEND_SRC_OVER, sampler: int = 0):
        self.cmd(CMD_DRAW_IMAGE_MESH, image, blend_mode | (sampler << 8),
                 (opacity, float(mesh), 0, 0, 0, 0))

    def cmd(self, op, a=0, b=0, m=(0, 0, 0, 0, 0, 0)):
        self.cmds.append((op, a, b, tuple(float(v) for v in m)))

    def to_bytes(self) -> bytes:
        verbs = bytearray()
        pts = []
        stops = []
        path_recs = []
        npts = 0
        for p in self.paths:
            pa = np.asarray(p.points, dtype=np.float32).reshape(-1, 2)
            path_recs.append(struct.pack("<5I", len(verbs), len(p.verbs), npts,
                                         len(pa), p.fill_rule | (PATH_APPENDED if p.appended else 0)))
            verbs.extend(bytes(p.verbs))
            pts.append(pa)
            npts += len(pa)
        paint_recs = []
        for q in self.paints:
            paint_recs.append(struct.pack(
                "<IIfIIII4fIIf", q.style, q.color & 0xFFFFFFFF, q.thickness,
                q.join, q.cap, q.blend_mode, q.shader, *[float(v) for v in q.g],
                len(stops), len(q.stops), float(q.feather)))
            stops.extend(q.stops)
        cmd_recs = [struct.pack("<3I6f", op, a, b, *m) for (op, a, b, m) in self.cmds]
        header = struct.pack("<12I", MAGIC, self.width, self.height,
                             self.clear_color & 0xFFFFFFFF, len(self.paths),
                             len(self.paints), len(self.cmds), len(verbs), npts,
                             len(stops), self.dither_mode, self.flags)
        vpad = bytes((4 - len(verbs) % 4) % 4)
        pts_bytes = (np.concatenate(pts).astype("<f4").tobytes()
                     if pts else b"")
        stop_bytes = b"".join(struct.pack("<fI", float(s), c & 0xFFFFFFFF)
                              for s, c in stops)
        image_bytes = b""
        if self.images or self.meshes:
            image_bytes = struct.pack("<2I", IMAGES_MAGIC, len(self.images))
            for im in self.images:
                a = np.ascontiguousarray(im.rgba, dtype=np.uint8)
                image_bytes += struct.pack("<2I", a.shape[1], a.shape[0]) + a.tobytes()
        mesh_bytes = b""
        if self.meshes:
            mesh_bytes = struct.pack("<2I", MESHES_MAGIC, len(self.meshes))
            for m in self.meshes:
                xy = np.ascontiguousarray(m.xy, dtype="<f4").reshape(-1, 2)
                uv = np.ascontiguousarray(m.uv, dtype="<f4").reshape(-1, 2)
                ix = np.ascontiguousarray(m.indices, dtype="<u2").reshape(-1)
                assert len(xy) == len(uv) and len(ix) % 3 == 0
                ib = ix.tobytes()
                mesh_bytes += (struct.pack("<2I", len(xy), len(ix)) + xy.tobytes() + uv.tobytes()
                               + ib + bytes((4 - len(ib) % 4) % 4))
        return (header + b"".join(path_recs) + b"".join(paint_recs)
                + b"".join(cmd_recs) + bytes(verbs) + vpad + pts_bytes + stop_bytes
                + image_bytes + mesh_bytes)

    @property
    def draw_count(self):
        return sum(1 for c in self.cmds if c[0] == CMD_DRAW_PATH)


def color_int(r, g, b, a) -> int:
    """Packs unit floats into rive::ColorInt 0xAARRGGBB (round to nearest)."""
    q = [int(round(float(v) * 255.0)) for v in (a, r, g, b)]
    return (q[0] << 24) | (q[1] << 16) | (q[2] << 8) | q[3]


def _random_color(rng, alpha_lo=0.5, alpha_hi=1.0):
    r, g, b = rng.uniform(0.0, 1.0, 3)
    a = rng.uniform(alpha_lo, alpha_hi)
    return color_int(r, g, b, a)


def _closed_cubic_contour(rng, ncubics, lo, hi):
    """One contour: move + ncubics cubics returning to the start + close."""
    p0 = rng.uniform(lo, hi, 2)
    pts = [p0]
    verbs = [VERB_MOVE]
    for i in range(ncubics):
        c = rng.uniform(lo, hi, (3, 2))
        if i == ncubics - 1:
            c[2] = p0
        pts.extend(c)
        verbs.append(VERB_CUBIC)
    verbs.append(VERB_CLOSE)
    return verbs, pts


def _open_cubic_contour(rng, ncubics, lo, hi):
    pts = [rng.uniform(lo, hi, 2)]
    verbs = [VERB_MOVE]
    for _ in range(ncubics):
        pts.extend(rng.uniform(lo, hi, (3, 2)))
        verbs.append(VERB_CUBIC)
    return verbs, pts


def plain_small(seed: int = 1, width: int = 512, height: int = 512,
                n_paths: int = 200, cubics: int = 8) -> Scene:
    """The plain small workload (512x512, 200 closed 8-cubic fills)."""
    rng = np.random.default_rng(seed)
    sc = Scene(width, height, clear_color=0xFFFFFFFF)
    for _ in range(n_paths):
        verbs, pts = _closed_cubic_contour(rng, cubics, 0.0, float(min(width, height)))
        pi = sc.add_path(Path(verbs, np.array(pts, np.float32), FILL_NONZERO))
        qi = sc.add_paint(Paint(style=STYLE_FILL, color=_random_color(rng)))
        sc.cmd(CMD_DRAW_PATH, pi, qi)
    return sc


def plain_canvas(rng, width: int, height: int, n_paths: int, cubics: int = 8) -> Scene:
    """The plain path distribution on a width x height canvas: closed
    single-contour fills of `cubics` cubics with every control point uniform
    over the canvas, nonzero, identity transform, solid colours (RGB uniform,
    alpha uniform in [0.5, 1]), srcOver, cleared to opaque white."""
    sc = Scene(width, height, clear_color=0xFFFFFFFF)
    ext = np.array([width, height], np.float64)
    for _ in range(n_paths):
        p0 = rng.uniform(0.0, 1.0, 2) * ext
        pts = [p0]
        verbs = [VERB_MOVE]
        for i in range(cubics):
            c = rng.uniform(0.0, 1.0, (3, 2)) * ext
            if i == cubics - 1:
                c[2] = p0
            pts.extend(c)
            verbs.append(VERB_CUBIC)
        verbs.append(VERB_CLOSE)
        pi = sc.add_path(Path(verbs, np.array(pts, np.float32), FILL_NONZERO))
        qi = sc.add_paint(Paint(style=STYLE_FILL, color=_random_color(rng)))
        sc.cmd(CMD_DRAW_PATH, pi, qi)
    return sc


def batched_scenes(seed: int = 3, count: int = 256, size_range=(256, 1920),
                   paths_median: float = 400.0, paths_sigma: float = 1.0,
                   paths_range=(50, 3000)):
    """The batched workload: `count` independent scenes with the plain path
    distribution; width and height independently log-uniform in size_range,
    path count lognormal(ln paths_median, paths_sigma) clipped to paths_range."""
    rng = np.random.default_rng(seed)
    lo, hi = math.log(size_range[0]), math.log(size_range[1])
    scenes = []
    for _ in range(count):
        w = int(round(math.exp(rng.uniform(lo, hi))))
        h = int(round(math.exp(rng.uniform(lo, hi))))
        n = int(np.clip(round(rng.lognormal(math.log(paths_median), paths_sigma)),
                        paths_range[0], paths_range[1]))
        scenes.append(plain_canvas(rng, w, h, n))
    return scenes


def _random_affine(rng, width, height, scale_range=(0.25, 4.0)):
    theta = rng.uniform(0.0, 2.0 * math.pi)
    s = math.exp(rng.uniform(math.log(scale_range[0]), math.log(scale_range[1])))
    tx = rng.uniform(0.0, width)
    ty = rng.uniform(0.0, height)
    c, sn = math.cos(theta) * s, math.sin(theta) * s
    return (c, sn, -sn, c, tx, ty)


def _gradient_paint(rng, paint: Paint):
    h = LOCAL_HALF_EXTENT
    nstops = int(rng.integers(2, 9))
    pos = np.sort(rng.uniform(0.0, 1.0, nstops)).astype(np.float32)
    pos[0] = 0.0 if rng.uniform() < 0.5 else pos[0]
    cols = [_random_color(rng) for _ in range(nstops)]
    if rng.uniform() < 0.5:
        paint.shader = SHADER_LINEAR
        a = rng.uniform(-h, h, 2)
        b = rng.uniform(-h, h, 2)
        paint.g = (a[0], a[1], b[0], b[1])
    else:
        paint.shader = SHADER_RADIAL
        c = rng.uniform(-h, h, 2)
        paint.g = (c[0], c[1], rng.uniform(h * 0.2, h * 2.0), 0.0)
    paint.stops = [(float(p), c) for p, c in zip(pos, cols)]


def full_feature(seed: int = 2, width: int = 2048, height: int = 2048,
                 n_paths: int = 5000, max_contours: int = 4,
                 min_cubics: int = 4, max_cubics: int = 64,
                 p_fill: float = 0.6, p_gradient: float = 0.3,
                 p_blend: float = 0.1, p_clip: float = 0.1,
                 scale_range=(0.25, 4.0)) -> Scene:
    """The full-feature single scene (defaults: 2048x2048, 5,000 paths)."""
    rng = np.random.default_rng(seed)
    sc = Scene(width, height, clear_color=0xFFFFFFFF)
    h = LOCAL_HALF_EXTENT
    for _ in range(n_paths):
        is_fill = rng.uniform() < p_fill
        ncont = int(rng.integers(1, max_contours + 1))
        verbs, pts = [], []
        for _c in range(ncont):
            nc = int(rng.integers(min_cubics, max_cubics + 1))
            if is_fill:
                v, p = _closed_cubic_contour(rng, nc, -h, h)
            else:
                v, p = _open_cubic_contour(rng, nc, -h, h)
            verbs += v
            pts += p
        fill_rule = FILL_EVENODD if (is_fill and rng.uniform() < 0.5) else FILL_NONZERO
        pi = sc.add_path(Path(verbs, np.array(pts, np.float32), fill_rule))
        paint = Paint(style=STYLE_FILL if is_fill else STYLE_STROKE,
                      color=_random_color(rng))
        if not is_fill:
            paint.thickness = float(np.exp(rng.normal(math.log(4.0), 0.7)))
            paint.join = int(rng.integers(0, 3))
            paint.cap = int(rng.integers(0, 3))
        if rng.uniform() < p_gradient:
            _gradient_paint(rng, paint)
        if rng.uniform() < p_blend:
            paint.blend_mode = int(BLEND_MODES[int(rng.integers(0, 16))])
        qi = sc.add_paint(paint)
        m = _random_affine(rng, width, height, scale_range)
        clipped = rng.uniform() < p_clip
        sc.cmd(CMD_SAVE)
        sc.cmd(CMD_TRANSFORM, m=m)
        if clipped:
            depth = int(rng.integers(1, 4))
            for _d in range(depth):
                v, p = _closed_cubic_contour(rng, int(rng.integers(3, 9)), -h * 1.2, h * 1.2)
                ci = sc.add_path(Path(v, np.array(p, np.float32), FILL_NONZERO))
                sc.cmd(CMD_CLIP_PATH, ci)
        sc.cmd(CMD_DRAW_PATH, pi, qi)
        sc.cmd(CMD_RESTORE)
    return sc


def stroke_stress(seed: int = 4, width: int = 1024, height: int = 1024,
                  n_strokes: int = 5000) -> Scene:
    """Tessellation-heavy strokes: 1-16 cubics, 20% cusp/near-degenerate."""
    rng = np.random.default_rng(seed)
    sc = Scene(width, height, clear_color=0xFFFFFFFF)
    for _ in range(n_strokes):
        n = int(rng.integers(1, 17))
        cx, cy = rng.uniform(0, width), rng.uniform(0, height)
        span = rng.uniform(8.0, 160.0)
        p = np.array([cx, cy]) + rng.uniform(-span, span, 2)
        pts = [p]
        verbs = [VERB_MOVE]
        for _k in range(n):
            p3 = np.array([cx, cy]) + rng.uniform(-span, span, 2)
            if rng.uniform() < 0.2:
                kind = int(rng.integers(0, 3))
                chord = p3 - p
                if kind == 0:   # inner points within 0.1 px of the chord
                    t = rng.uniform(0, 1, 2)
                    nrm = np.array([-chord[1], chord[0]])
                    nrm = nrm / max(np.linalg.norm(nrm), 1e-6)
                    p1 = p + chord * t[0] + nrm * rng.uniform(-0.1, 0.1)
                    p2 = p + chord * t[1] + nrm * rng.uniform(-0.1, 0.1)
                elif kind == 1:  # coincident with the endpoints
                    p1, p2 = p.copy(), p3.copy()
                else:           # cusp: control points crossed over
                    p1, p2 = p3 + (p3 - p) * 0.5, p - (p3 - p) * 0.5
            else:
                p1 = np.array([cx, cy]) + rng.uniform(-span, span, 2)
                p2 = np.array([cx, cy]) + rng.uniform(-span, span, 2)
            pts += [p1, p2, p3]
            verbs.append(VERB_CUBIC)
            p = p3
        pi = sc.add_path(Path(verbs, np.array(pts, np.float32), FILL_NONZERO))
        r, g, b = rng.uniform(0, 1, 3)
        width_px = float(math.exp(rng.uniform(math.log(0.5), math.log(64.0))))
        qi = sc.add_paint(Paint(style=STYLE_STROKE, color=color_int(r, g, b, 0.8),
                                thickness=width_px, join=JOIN_ROUND, cap=CAP_ROUND))
        sc.cmd(CMD_DRAW_PATH, pi, qi)
    return sc


def feathered_strokes(seed: int = 31, width: int = 320, height: int = 256, n_paths: int = 40,
                      p_feather: float = 0.6, feather_range=(0.5, 8.0)) -> Scene:
    """The full-feature distributions with a share of the strokes feathered
    (RenderPaint::feather uniform in `feather_range`). Transforms scale by at
    most 2, so every feather stays below the 32-pixel radius at which the
    reference switches to its feather atlas: radius = 1.5 x feather x scale."""
    sc = full_feature(seed=seed, width=width, height=height, n_paths=n_paths, max_cubics=10,
                      p_fill=0.4, p_clip=0.15, scale_range=(0.5, 2.0))
    rng = np.random.default_rng(seed + 1)
    for p in sc.paints:
        if p.style == STYLE_STROKE and rng.uniform() < p_feather:
            p.feather = float(rng.uniform(*feather_range))
    return sc


def feathered(seed: int = 33, width: int = 320, height: int = 256, n_paths: int = 40,
              p_feather: float = 0.6, feather_range=(0.5, 8.0)) -> Scene:
    """The full-feature distributions with a share of the fills and strokes
    feathered. The reference draws feathered fills only with the clockwise fill
    rule, so the feathered fills' paths are clockwise. Transforms scale by at
    most 2, keeping every feather below the 32-pixel radius of the feather
    atlas (radius = 1.5 x feather x scale)."""
    sc = full_feature(seed=seed, width=width, height=height, n_paths=n_paths, max_cubics=10,
                      p_fill=0.7, p_clip=0.15, scale_range=(0.5, 2.0))
    rng = np.random.default_rng(seed + 1)
    for op, a, b, _ in sc.cmds:
        if op != CMD_DRAW_PATH:
            continue
        paint = sc.paints[b]
        if rng.uniform() < p_feather:
            paint.feather = float(rng.uniform(*feather_range))
            if paint.style == STYLE_FILL:
                sc.paths[a].fill_rule = FILL_CLOCKWISE
    return sc


def feathered_atlas(seed: int = 35, width: int = 384, height: int = 320, n_paths: int = 36,
                    p_feather: float = 0.7, feather_range=(4.0, 40.0)) -> Scene:
    """Wide feathers: the full-feature distributions with a share of the fills
    and strokes feathered by up to 40 (radius = 1.5 x feather x scale, scale
    0.5..2), so many reach the 32-pixel radius at which the reference renders
    them through its feather atlas at half resolution or less
    (draw.cpp:387-404), beside feathers drawn directly. Feathered fills are
    clockwise, as the reference draws them."""
    sc = full_feature(seed=seed, width=width, height=height, n_paths=n_paths, max_cubics=10,
                      p_fill=0.65, p_clip=0.15, scale_range=(0.5, 2.0))
    rng = np.random.default_rng(seed + 1)
    for op, a, b, _ in sc.cmds:
        if op != CMD_DRAW_PATH:
            continue
        paint = sc.paints[b]
        if rng.uniform() < p_feather:
            paint.feather = float(rng.uniform(*feather_range))
            if paint.style == STYLE_FILL:
                sc.paths[a].fill_rule = FILL_CLOCKWISE
    return sc


def _procedural_image(rng, w: int, h: int) -> Image:
    """A w x h test image: a two-colour checker under a diagonal gradient with
    a soft transparent disc, premultiplied RGBA8."""
    y, x = np.mgrid[0:h, 0:w].astype(np.float32)
    cell = float(rng.integers(2, 9))
    check = ((np.floor(x / cell) + np.floor(y / cell)) % 2)[..., None]
    c0, c1 = rng.uniform(0, 1, 3), rng.uniform(0, 1, 3)
    rgb = c0 * (1 - check) + c1 * check
    t = ((x / max(w - 1, 1) + y / max(h - 1, 1)) * .5)[..., None]
    rgb = rgb * (1 - .5 * t) + rng.uniform(0, 1, 3) * (.5 * t)
    cx, cy, r = w * rng.uniform(.3, .7), h * rng.uniform(.3, .7), min(w, h) * rng.uniform(.2, .45)
    d = np.sqrt((x - cx) ** 2 + (y - cy) ** 2)
    a = np.clip(.35 + (d - r) / max(r * .5, 1.0), .35, 1.0)[..., None]
    rgba = np.concatenate([rgb * a, a], -1)
    return Image(np.clip(np.rint(rgba * 255), 0, 255).astype(np.uint8))


def images(seed: int = 41, width: int = 384, height: int = 320, n_images: int = 6,
           n_draws: int = 24, n_paths: int = 16) -> Scene:
    """Images drawn with Renderer::drawImage between full-feature paths: each of
    `n_images` procedural images (power-of-two and odd sizes, 7..200 px)
    drawn under random affine transforms (magnified and minified, so the mip
    chain is sampled), with every ImageSampler (bilinear / nearest, clamp /
    repeat / mirror), opacity in [0.3, 1], some with advanced blend modes and
    some under clip paths."""
    rng = np.random.default_rng(seed)
    sc = full_feature(seed=seed, width=width, height=height, n_paths=n_paths, max_cubics=8,
                      p_clip=0.2, scale_range=(0.5, 2.0))
    sizes = [(64, 64), (128, 32), (7, 13), (200, 90), (33, 33), (16, 128)]
    for k in range(n_images):
        w, h = sizes[k % len(sizes)]
        sc.add_image(_procedural_image(rng, w, h))
    clip_paths = [i for i, _ in enumerate(sc.paths)]
    for k in range(n_draws):
        im = int(rng.integers(0, n_images))
        w, h = sc.images[im].rgba.shape[1], sc.images[im].rgba.shape[0]
        # Target size 12..260 px along the longer side, rotated.
        target = float(np.exp(rng.uniform(np.log(12), np.log(260))))
        s = target / max(w, h)
        th = rng.uniform(0, 2 * np.pi)
        c, sn = np.cos(th) * s, np.sin(th) * s
        tx, ty = rng.uniform(0, width), rng.uniform(0, height)
        sc.cmd(CMD_SAVE)
        sc.cmd(CMD_TRANSFORM, m=(c, sn, -sn, c, tx - (c * w - sn * h) / 2,
                                 ty - (sn * w + c * h) / 2))
        if clip_paths and rng.uniform() < 0.2:
            sc.cmd(CMD_CLIP_PATH, int(rng.choice(clip_paths)))
        blend = int(rng.choice(BLEND_MODES)) if rng.uniform() < 0.25 else BLEND_SRC_OVER
        sampler = sampler_key(int(rng.integers(0, 3)), int(rng.integers(0, 3)),
                              int(rng.integers(0, 2)))
        sc.draw_image(im, float(rng.uniform(0.3, 1.0)), blend, sampler)
        sc.cmd(CMD_RESTORE)
    return sc


def _grid_mesh(rng, w: float, h: float, gx: int, gy: int, uv_scale: float, warp: float) -> Mesh:
    """A (gx x gy)-cell grid over [0, w] x [0, h], its inner vertices moved by
    up to `warp` cells, texture coordinates (i / gx, j / gy) * uv_scale; two
    triangles per cell, alternating diagonals (both windings occur)."""
    jj, ii = np.meshgrid(np.arange(gy + 1), np.arange(gx + 1), indexing="ij")
    x = ii * (w / gx)
    y = jj * (h / gy)
    inner = (ii > 0) & (ii < gx) & (jj > 0) & (jj < gy)
    x = x + inner * rng.uniform(-warp, warp, x.shape) * (w / gx)
    y = y + inner * rng.uniform(-warp, warp, y.shape) * (h / gy)
    xy = np.stack([x.ravel(), y.ravel()], 1).astype(np.float32)
    uv = (np.stack([(ii / gx).ravel(), (jj / gy).ravel()], 1) * uv_scale).astype(np.float32)
    idx = []
    for j in range(gy):
        for i in range(gx):
            a, b = j * (gx + 1) + i, j * (gx + 1) + i + 1
            c, d = a + gx + 1, b + gx + 1
            if (i + j) % 2:
                idx += [a, b, d, a, d, c]
            else:
                idx += [a, b, c, b, d, c]
    return Mesh(xy, uv, np.array(idx, np.uint16))


def _soup_mesh(rng, w: float, h: float, n_tris: int) -> Mesh:
    """`n_tris` random triangles over [0, w] x [0, h] that overlap one another
    (every covering triangle blends), random windings and texture coordinates
    in [-0.5, 1.5], some vertices shared."""
    nv = max(3, int(n_tris * 1.5))
    xy = np.stack([rng.uniform(0, w, nv), rng.uniform(0, h, nv)], 1).astype(np.float32)
    uv = rng.uniform(-0.5, 1.5, (nv, 2)).astype(np.float32)
    idx = rng.integers(0, nv, (n_tris, 3)).astype(np.uint16)
    return Mesh(xy, uv, idx.ravel())


def image_meshes(seed: int = 43, width: int = 384, height: int = 320, n_images: int = 5,
                 n_draws: int = 22, n_paths: int = 14) -> Scene:
    """Image meshes drawn with Renderer::drawImageMesh between full-feature
    paths: warped grids (texture coordinates up to 2.5, so repeat and mirror
    wrap) and overlapping triangle soups, magnified and minified under
    rotations (so the implicit level of detail picks different mip levels),
    with every ImageSampler, opacity in [0.3, 1], some advanced blend modes,
    some under clip paths and some under axis-aligned rectangle clips (clip
    rects); a few drawImage rectangles too."""
    rng = np.random.default_rng(seed)
    sc = full_feature(seed=seed, width=width, height=height, n_paths=n_paths, max_cubics=8,
                      p_clip=0.2, scale_range=(0.5, 2.0))
    sizes = [(64, 64), (128, 32), (9, 15), (200, 90), (33, 33)]
    for k in range(n_images):
        w, h = sizes[k % len(sizes)]
        sc.add_image(_procedural_image(rng, w, h))
    clip_paths = [i for i, _ in enumerate(sc.paths)]
    # Axis-aligned rectangles: clipPath turns these into clip rects.
    rects = []
    for _ in range(3):
        x0, y0 = rng.uniform(0, width * .6), rng.uniform(0, height * .6)
        x1, y1 = x0 + rng.uniform(40, width * .5), y0 + rng.uniform(40, height * .5)
        pts = np.array([[x0, y0], [x1, y0], [x1, y1], [x0, y1]], np.float32)
        rects.append(sc.add_path(Path([VERB_MOVE, VERB_LINE, VERB_LINE, VERB_LINE, VERB_CLOSE],
                                      pts, FILL_NONZERO)))
    for k in range(n_draws):
        im = int(rng.integers(0, n_images))
        iw, ih = sc.images[im].rgba.shape[1], sc.images[im].rgba.shape[0]
        if rng.uniform() < 0.6:
            mesh = _grid_mesh(rng, float(iw), float(ih), int(rng.integers(1, 7)),
                              int(rng.integers(1, 6)), float(rng.choice([1.0, 1.0, 2.5])),
                              float(rng.uniform(0, .35)))
        else:
            mesh = _soup_mesh(rng, float(iw), float(ih), int(rng.integers(2, 12)))
        mi = sc.add_mesh(mesh)
        target = float(np.exp(rng.uniform(np.log(10), np.log(300))))
        s = target / max(iw, ih)
        th = rng.uniform(0, 2 * np.pi)
        c, sn = np.cos(th) * s, np.sin(th) * s
        tx, ty = rng.uniform(0, width), rng.uniform(0, height)
        sc.cmd(CMD_SAVE)
        r = rng.uniform()
        if r < 0.15:
            sc.cmd(CMD_CLIP_PATH, int(rng.choice(rects)))
        elif r < 0.3 and clip_paths:
            sc.cmd(CMD_CLIP_PATH, int(rng.choice(clip_paths)))
        sc.cmd(CMD_TRANSFORM, m=(c, sn, -sn, c, tx - (c * iw - sn * ih) / 2,
                                 ty - (sn * iw + c * ih) / 2))
        blend = int(rng.choice(BLEND_MODES)) if rng.uniform() < 0.25 else BLEND_SRC_OVER
        sampler = sampler_key(int(rng.integers(0, 3)), int(rng.integers(0, 3)),
                              int(rng.integers(0, 2)))
        opacity = float(rng.uniform(0.3, 1.0))
        if k % 7 == 3:
            sc.draw_image(im, opacity, blend, sampler)
        else:
            sc.draw_image_mesh(im, mi, opacity, blend, sampler)
        sc.cmd(CMD_RESTORE)
    return sc


def mesh_overlap(opacity: float = 0.5) -> Scene:
    """Two overlapping triangles of one image mesh, one clockwise and one
    counterclockwise, textured by an opaque red 4x4 image with a nearest
    sampler, at `opacity` on white without dither: where both cover a pixel
    it blends twice."""
    sc = Scene(64, 64, clear_color=0xFFFFFFFF, dither_mode=0)
    rgba = np.zeros((4, 4, 4), np.uint8)
    rgba[..., 0] = 255
    rgba[..., 3] = 255
    sc.add_image(Image(rgba))
    xy = np.array([[8, 8], [56, 8], [8, 56], [16, 16], [16, 60], [60, 16]], np.float32)
    uv = np.array([[0, 0], [1, 0], [0, 1], [0, 0], [0, 1], [1, 0]], np.float32)
    sc.add_mesh(Mesh(xy, uv, np.arange(6, dtype=np.uint16)))
    sc.draw_image_mesh(0, 0, opacity, BLEND_SRC_OVER, sampler_key(filt=FILTER_NEAREST))
    return sc
