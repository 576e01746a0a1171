"""The deferred command-stream reader (rive_runtime_gb300.cmdbuf) against the
reference's own consumer of the stream, replayRenderCommands.

* Stored sessions (tests/golden/cmdbuf): recorded .riv animations as the
  reference's DeferredFactory records them, frame after frame; frame k read by
  the reader and planned by the planner equals the reference's replay of it,
  byte for byte (runs anywhere).
* Where the reference sources exist: the wire layout (POD sizes, opcode
  numbers) is checked against its headers, every golden scene round-trips
  through its recorder, and crafted streams exercise what recorded content
  does not (destroys and id reuse, transformed addRenderPath, versions named
  by later draws, canvas brackets, shader clears).
"""
import glob
import os
import shutil
import struct
import subprocess
import tempfile

import numpy as np
import pytest

from conftest import golden_names, load_golden, load_package
from planner_compare import diff_captures
import oracle

load_package()
from rive_runtime_gb300 import capture, cmdbuf, scene  # noqa: E402
from inputgen import planner  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
SESSIONS = os.path.join(HERE, "golden", "cmdbuf")
REF = oracle.reference_available()


def _session_frames():
    out = []
    for cap in sorted(glob.glob(os.path.join(SESSIONS, "*_f*.cap"))):
        base = os.path.basename(cap)[:-4]
        name, k = base.rsplit("_f", 1)
        out.append((name, int(k)))
    return out


@pytest.mark.parametrize("name,k", _session_frames())
def test_session_frame_plans_like_the_reference_replay(name, k):
    with open(os.path.join(SESSIONS, name + ".rcs"), "rb") as f:
        data = f.read()
    with open(os.path.join(SESSIONS, f"{name}_f{k}.cap"), "rb") as f:
        want = capture.parse(f.read())
    sc, st = cmdbuf.rcs_frame_scene(data, k)
    assert st.dropped_unresolved == 0
    assert diff_captures(want, planner.plan(sc.to_bytes())) == []


def test_session_files_parse():
    for path in glob.glob(os.path.join(SESSIONS, "*.rcs")):
        with open(path, "rb") as f:
            frames, hdr = cmdbuf.read_rcs(f.read())
        assert len(frames) > 1 and hdr["width"] > 0


def test_malformed_streams_are_refused():
    with pytest.raises(cmdbuf.CmdbufError, match="opcode"):
        cmdbuf.command_buffer_scene(bytes([200]), b"", 8, 8)
    with pytest.raises(cmdbuf.CmdbufError, match="overrun"):
        cmdbuf.command_buffer_scene(bytes([cmdbuf.OP["drawPath"], 1, 2]), b"", 8, 8)
    with pytest.raises(cmdbuf.CmdbufError, match="skips ahead"):
        cmdbuf.command_buffer_scene(bytes([cmdbuf.OP["makePaint"]]) + struct.pack("<II", 5, 0),
                                    b"", 8, 8)
    with pytest.raises(cmdbuf.CmdbufError):
        cmdbuf.read_rcs(b"RCS1" + bytes(10))


# ---------------------------------------------------------------------------
# Against the reference's sources.

_PROBE = r"""
#include "rive/renderer/cmd/render_commands.hpp"
#include <cstdio>
using namespace rive::cmd;
int main() {
#define P(cmd, POD) printf("%s %d %zu\n", #cmd, (int)RenderCmd::cmd, payloadSizeOf(RenderCmd::cmd));
    RIVE_RENDER_CMD_TABLE(P)
    printf("last %d\n", (int)RenderCmd::lastRenderCmd);
}
"""


@pytest.mark.skipif(not REF or shutil.which("g++") is None, reason="reference sources absent")
def test_wire_layout_matches_the_reference_headers():
    ref = oracle.REFERENCE_SOURCES
    with tempfile.TemporaryDirectory() as td:
        src, exe = os.path.join(td, "probe.cpp"), os.path.join(td, "probe")
        with open(src, "w") as f:
            f.write(_PROBE)
        subprocess.check_call(["g++", "-std=c++17", "-w", f"-I{ref}/include",
                               f"-I{ref}/renderer/include", src, "-o", exe])
        out = subprocess.check_output([exe], text=True).split("\n")
    seen = {}
    for line in out:
        parts = line.split()
        if len(parts) == 3:
            seen[parts[0]] = (int(parts[1]), int(parts[2]))
        elif len(parts) == 2:
            assert int(parts[1]) == len(cmdbuf.OPCODES) - 1
    assert set(seen) == set(cmdbuf.OPCODES)
    for name, (op, size) in seen.items():
        fmt = cmdbuf.POD_FORMATS[name]
        assert cmdbuf.OP[name] == op, name
        assert (struct.calcsize(fmt) if fmt else 0) == size, name


@pytest.mark.skipif(not REF, reason="reference sources absent")
@pytest.mark.parametrize("name", golden_names())
def test_recorded_golden_scene_reads_back(name):
    """Scene -> the reference's recorder -> stream -> the reader -> scene:
    planned and captured, it equals the reference's replay of the stream."""
    cap, sb = load_golden(name)
    if cap.textures:
        pytest.skip("image draws: the command-buffer reader leaves them out")
    rcb = oracle.cmdbuf_record(sb)
    want = capture.parse(oracle.cmdbuf_replay(rcb))
    sc, st = cmdbuf.rcb_scene(rcb, keep_feathered=True)
    assert diff_captures(want, capture.parse(oracle.reference_capture(sc.to_bytes()))) == []
    feathered = any(p.feather for p in sc.paints)
    if not sc.flags & scene.FLAG_TRIANGULATE and not feathered:
        assert diff_captures(want, planner.plan(sc.to_bytes())) == []


class _Stream:
    """A crafted command stream (the reference's wire layout)."""

    def __init__(self):
        self.cmds = bytearray()
        self.blobs = bytearray()

    def blob(self, data: bytes) -> int:
        self.blobs += bytes((-len(self.blobs)) % 8)
        off = len(self.blobs)
        self.blobs += data
        return off

    def op(self, name, *fields):
        self.cmds.append(cmdbuf.OP[name])
        fmt = cmdbuf.POD_FORMATS[name]
        if fmt:
            self.cmds += struct.pack(fmt, *fields)
        return self

    def raw(self, verbs, pts):
        vo = self.blob(bytes(verbs))
        po = self.blob(np.asarray(pts, "<f4").tobytes())
        return vo, po, len(verbs), len(pts)

    def make_path(self, rid, gen, verbs, pts, fill=0):
        vo, po, nv, npt = self.raw(verbs, pts)
        return self.op("makePath", rid, gen, vo, po, nv, npt, fill, 0)

    def rcb(self, w, h, clear=0xFF202028):
        return struct.pack("<6IQQ", cmdbuf.RCB_MAGIC, w, h, clear, 1, 0, len(self.cmds),
                           len(self.blobs)) + bytes(self.cmds) + bytes(self.blobs)


M, L, C, Z = scene.VERB_MOVE, scene.VERB_LINE, scene.VERB_CUBIC, scene.VERB_CLOSE
INVALID = 0xFFFFFFFF


def _crafted():
    s = _Stream()
    # Path 0 through makeRenderPath (pruned: the repeated point is dropped).
    s.make_path(0, 0, [M, L, L, L, L, Z], [(20, 20), (120, 30), (120, 30), (110, 140), (30, 120)])
    # Path 1: empty, clockwise, appended; then a transformed copy of path 0
    # whose collapsed segments are pruned after the transform.
    s.op("makeEmptyPath", 1, 0).op("pathFillRule", 1, scene.FILL_CLOCKWISE)
    vo, po, nv, npt = s.raw([M, C, L, Z], [(150, 40), (200, 10), (240, 90), (210, 150),
                                            (160, 140)])
    s.op("pathAddRawPath", vo, po, 1, nv, npt, 0)
    s.op("pathAddRenderPath", 1, 0, 1.0, 0.0, 0.0, 0.25, 130.0, 150.0)
    s.op("pathAddRenderPath", 1, 0, 0.5, 0.0, 0.0, 0.0, 10.0, 200.0)  # collapses to lines
    # Paints and a gradient.
    s.op("makePaint", 0, 0).op("paintColor", 0, 0xFFE04040)
    s.op("makePaint", 1, 0).op("paintStyle", 1, 0).op("paintThickness", 1, 6.0)
    s.op("paintJoin", 1, 1).op("paintCap", 1, 1)
    co = s.blob(struct.pack("<2I", 0xFF00E0A0, 0xFFE000A0))
    so = s.blob(struct.pack("<2f", 0.0, 1.0))
    s.op("makeLinearGradient", 0, 0, 0.0, 0.0, 256.0, 256.0, co, so, 2, 0)
    s.op("paintShader", 1, 0).op("paintShader", 1, INVALID).op("paintShader", 1, 0)
    s.op("save").op("transform", 1.0, 0.0, 0.0, 1.0, 4.0, 2.0)
    s.op("drawPath", 0, 0, 0, 0)
    s.op("drawPath", 1, 1, 0, 0)
    # A drawn paint mutated again: a new version; a later draw names the old.
    s.op("resourceNewVersion", cmdbuf.KIND_PAINT, 0, 1).op("paintColor", 0, 0xFF4060E0)
    s.op("drawPath", 1, 0, 0, 1)
    s.op("drawPath", 0, 0, 0, 0)  # the outgoing (red) version
    # A drawn path rewound and refilled under a new version.
    s.op("resourceNewVersion", cmdbuf.KIND_PATH, 1, 1).op("pathRewind", 1)
    vo, po, nv, npt = s.raw([M, L, L, Z], [(60, 160), (200, 170), (90, 240)])
    s.op("pathAddRawPath", vo, po, 1, nv, npt, 0)
    s.op("modulateOpacity", 0.5).op("drawPath", 1, 0, 1, 1).op("restore")
    # Destroy and retake id 0 with a new generation; a stale destroy no-ops.
    s.op("destroyResource", cmdbuf.KIND_PATH, 0, 0)
    s.op("drawPath", 0, 0, 0, 1)  # unresolved: dropped
    s.make_path(0, 1, [M, L, L, Z], [(180, 180), (250, 200), (200, 250)])
    s.op("destroyResource", cmdbuf.KIND_PATH, 0, 0)
    # Clip and draw.
    s.op("save").op("clipPath", 1, 1).op("drawPath", 0, 1, 0, 0).op("restore")
    # Canvas content needs a host canvas: the bare replay drops it.
    s.op("canvasContentBegin", 0x80000001, 0xFFFFFFFF).op("drawPath", 0, 0, 0, 1)
    s.op("canvasContentEnd", 0x80000001)
    s.op("drawImage", 7, 0, 0, 1, 3, 1.0)  # unknown image: dropped
    s.op("paintInvalidateStroke", 1)
    return s


@pytest.mark.skipif(not REF, reason="reference sources absent")
def test_crafted_stream_matches_the_reference_replay():
    rcb = _crafted().rcb(256, 256)
    want = capture.parse(oracle.cmdbuf_replay(rcb))
    sc, st = cmdbuf.rcb_scene(rcb)
    assert st.dropped_unresolved == 1 and st.dropped_canvas == 1 and st.dropped_images == 1
    assert st.draws == 6
    assert diff_captures(want, capture.parse(oracle.reference_capture(sc.to_bytes()))) == []
    assert diff_captures(want, planner.plan(sc.to_bytes())) == []


@pytest.mark.gpu
@pytest.mark.parametrize("name,k", _session_frames())
def test_session_frame_renders_on_the_gpu(name, k):
    """Reader -> planner -> the CUDA flush, against the oracle on the
    reference's own replay of the frame."""
    from rive_runtime_gb300 import rive_cuda
    with open(os.path.join(SESSIONS, name + ".rcs"), "rb") as f:
        data = f.read()
    with open(os.path.join(SESSIONS, f"{name}_f{k}.cap"), "rb") as f:
        want = oracle.render(capture.parse(f.read()))
    sc, _ = cmdbuf.rcs_frame_scene(data, k)
    ctx = rive_cuda.Context(0)
    try:
        got = ctx.render(planner.plan(sc.to_bytes()))
    finally:
        ctx.close()
    d = np.abs(got.astype(np.int16) - want.astype(np.int16)).max(axis=2)
    assert float((d <= 2).mean()) >= 0.999 and int(d.max()) <= 8, (name, k)
