"""The .sriv renderer-call stream reader (rive_runtime_gb300.sriv): wire
format, resource state across frames, what is dropped, and, where the
reference sources exist, the planner against the reference front end on
frames of the reference's own recorded animations."""
import glob
import os
import struct

import numpy as np
import pytest

from conftest import load_package
from planner_compare import diff_captures
import oracle

load_package()
from rive_runtime_gb300 import capture, scene, sriv  # noqa: E402
from inputgen import planner  # noqa: E402


class _Writer:
    """A minimal encoder of the stream layout (varuints, little-endian f32)."""

    def __init__(self):
        self.b = bytearray(b"SRIV")
        self.u(1)

    def u(self, v):
        while True:
            c = v & 0x7F
            v >>= 7
            self.b.append(c | (0x80 if v else 0))
            if not v:
                return self

    def f(self, *vals):
        for v in vals:
            self.b += struct.pack("<f", v)
        return self

    def raw_path(self, pid, verbs, pts):
        self.u(sriv.OP_ADD_RAW_PATH).u(pid).u(len(verbs))
        for v in verbs:
            self.u(v)
        self.u(len(pts))
        for x, y in pts:
            self.f(x, y)
        return self


def _square(x0, y0, s):
    return [scene.VERB_MOVE, scene.VERB_LINE, scene.VERB_LINE, scene.VERB_LINE,
            scene.VERB_CLOSE], [(x0, y0), (x0 + s, y0), (x0 + s, y0 + s), (x0, y0 + s)]


def _two_frame_stream():
    w = _Writer()
    w.u(sriv.OP_FRAME_SIZE).u(64).u(48)
    w.u(sriv.OP_MAKE_RENDER_PATH).u(0)
    w.u(sriv.OP_FILL_RULE).u(0).u(scene.FILL_CLOCKWISE)
    w.raw_path(0, *_square(4, 4, 20))
    w.u(sriv.OP_MAKE_RENDER_PAINT).u(0)
    w.u(sriv.OP_COLOR).u(0).u(0xFF336699)
    w.u(sriv.OP_MAKE_LINEAR_GRADIENT).u(0).u(2).u(0xFF000000).f(0.0).u(0xFFFFFFFF).f(1.0)
    w.f(0, 0, 64, 0)
    w.u(sriv.OP_SAVE)
    w.u(sriv.OP_TRANSFORM).f(1, 0, 0, 1, 3, 2)
    w.u(sriv.OP_MODULATE_OPACITY).f(0.5)
    w.u(sriv.OP_DRAW_PATH).u(0).u(0)
    w.u(sriv.OP_RESTORE)
    w.u(sriv.OP_FRAME)
    # Frame 1: the path is rewound and re-filled, the paint gets shader id 0
    # (the gradient) and a second, feathered paint draws too (dropped).
    w.u(sriv.OP_REWIND).u(0)
    w.raw_path(0, *_square(10, 10, 30))
    w.u(sriv.OP_SHADER).u(0).u(0)
    w.u(sriv.OP_MAKE_RENDER_PAINT).u(1)
    w.u(sriv.OP_FEATHER).u(1).f(4.0)
    w.u(sriv.OP_DRAW_PATH).u(0).u(0)
    w.u(sriv.OP_DRAW_PATH).u(0).u(1)
    w.u(sriv.OP_DECODE_IMAGE).u(0).u(3)
    w.b += b"abc"
    w.u(sriv.OP_DRAW_IMAGE).u(0).u(3).f(1.0)
    return bytes(w.b)


def test_reads_frames_and_resource_state():
    st = sriv.read_sriv(_two_frame_stream())
    assert (st.width, st.height) == (64, 48) and len(st.frames) == 2

    sc0, s0 = st.frame_scene(0)
    assert s0.draws == 1 and s0.dropped_feathered == 0
    assert [c[0] for c in sc0.cmds] == [scene.CMD_SAVE, scene.CMD_TRANSFORM,
                                        scene.CMD_MODULATE_OPACITY, scene.CMD_DRAW_PATH,
                                        scene.CMD_RESTORE]
    assert sc0.cmds[1][3] == (1, 0, 0, 1, 3, 2) and sc0.cmds[2][3][0] == 0.5
    (p,) = sc0.paths
    assert p.fill_rule == scene.FILL_CLOCKWISE and p.verbs[0] == scene.VERB_MOVE
    assert np.allclose(p.points[2], (24, 24))
    (q,) = sc0.paints
    assert q.color == 0xFF336699 and q.shader == scene.SHADER_NONE

    sc1, s1 = st.frame_scene(1)
    assert s1.draws == 1 and s1.dropped_feathered == 1 and s1.dropped_images == 1
    (p,) = sc1.paths
    assert np.allclose(p.points[0], (10, 10))  # rewound, then the new square
    (q,) = sc1.paints
    assert q.shader == scene.SHADER_LINEAR and len(q.stops) == 2


def test_truncated_raw_path_keeps_the_verbs_that_have_points():
    w = _Writer()
    w.u(sriv.OP_FRAME_SIZE).u(8).u(8)
    w.u(sriv.OP_MAKE_RENDER_PATH).u(0)
    w.u(sriv.OP_ADD_RAW_PATH).u(0).u(3).u(scene.VERB_MOVE).u(scene.VERB_LINE)
    w.u(scene.VERB_CUBIC).u(2).f(0, 0, 1, 1)  # the cubic's points are missing
    w.u(sriv.OP_MAKE_RENDER_PAINT).u(0)
    w.u(sriv.OP_DRAW_PATH).u(0).u(0)
    sc, _ = sriv.read_sriv(bytes(w.b)).frame_scene(0)
    assert sc.paths[0].verbs == [scene.VERB_MOVE, scene.VERB_LINE]


def test_errors():
    with pytest.raises(sriv.SrivError):
        sriv.read_sriv(b"RIVE\x01")
    w = _Writer().u(sriv.OP_FRAME_SIZE).u(8).u(8).u(99)
    with pytest.raises(sriv.SrivError, match="opcode"):
        sriv.read_sriv(bytes(w.b))
    w = _Writer().u(sriv.OP_FRAME_SIZE).u(8).u(8).u(sriv.OP_DRAW_PATH).u(5).u(0)
    with pytest.raises(sriv.SrivError, match="unknown path"):
        sriv.read_sriv(bytes(w.b))
    w = _Writer().u(sriv.OP_SAVE)
    with pytest.raises(sriv.SrivError, match="frame size"):
        sriv.read_sriv(bytes(w.b))
    assert sriv.read_sriv(bytes(w.b), default_size=(16, 16)).width == 16
    with pytest.raises(sriv.SrivError, match="truncated"):
        sriv.read_sriv(_two_frame_stream()[:-3])


def test_planner_plans_converted_frames():
    """Clockwise fills, clip rects and modulated opacity go through the planner
    and the oracle."""
    sc, _ = sriv.read_sriv(_two_frame_stream()).frame_scene(0)
    cap = planner.plan(sc.to_bytes())
    (f,) = cap.flushes
    batches = np.asarray(f.batches).reshape(-1, 8)
    assert (batches[:, 5] & 2).all()  # gpu::ShaderMiscFlags::clockwiseFill
    img = oracle.render(cap)
    # 0x336699 at half of 0xFF alpha, drawn at (7..27, 6..26) over transparent.
    assert img[15, 15, 3] == 128 and img[2, 2, 3] == 0


SILVERS = os.path.join(oracle.REFERENCE_SOURCES, "tests", "unit_tests", "silvers")


@pytest.mark.skipif(not oracle.reference_available() or not os.path.isdir(SILVERS),
                    reason="reference sources absent")
def test_planner_matches_reference_on_recorded_animations():
    """Every 12th recorded animation, first and middle frame: the planner's
    records equal the reference front end's byte for byte."""
    files = sorted(glob.glob(os.path.join(SILVERS, "*.sriv")))[::12]
    checked = 0
    for path in files:
        with open(path, "rb") as fh:
            st = sriv.read_sriv(fh.read(), default_size=(500, 500))
        for k in sorted({0, len(st.frames) // 2}):
            sb = st.frame_scene(k)[0].to_bytes()
            ref = capture.parse(oracle.reference_capture(sb))
            assert diff_captures(ref, planner.plan(sb)) == [], (os.path.basename(path), k)
            checked += 1
    assert checked >= 20
