"""Regenerates the deferred command-stream fixtures in cmdbuf/.

Each cmdbuf/<name>.rcs is a session of the reference's deferred 2D command
buffer (renderer/include/rive/renderer/cmd/render_command_buffer.hpp): one of
its recorded .riv animations (tests/unit_tests/silvers/<name>.sriv) replayed by
its own replaySerializedCommands into its DeferredFactory, one command stream
per frame, resources kept across frames. cmdbuf/<name>_f<k>.cap is what the
reference's own replayRenderCommands makes of frame k (after consuming frames
0..k-1 for their resources) in front of the recording RenderContextImpl. Both
come from oracle/_ref/cmdbuf_capture (oracle/Makefile, target cmdbuf), so this
runs only where the reference sources exist:

    python tests/golden/make_cmdbuf.py
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))
import oracle  # noqa: E402

SESSIONS = ["component_list_grouped", "script_artboards_opacity", "juice"]


def frames_of(rcs_path):
    import struct
    with open(rcs_path, "rb") as f:
        return struct.unpack_from("<8I", f.read(32))[6]


def main():
    tool = oracle.build_cmdbuf_tool()
    silvers = os.path.join(oracle.REFERENCE_SOURCES, "tests", "unit_tests", "silvers")
    out = os.path.join(HERE, "cmdbuf")
    os.makedirs(out, exist_ok=True)
    for name in SESSIONS:
        rcs = os.path.join(out, name + ".rcs")
        subprocess.run([tool, "record-sriv", os.path.join(silvers, name + ".sriv"), rcs],
                       check=True)
        n = frames_of(rcs)
        for k in sorted({0, n // 2, n - 1}):
            subprocess.run([tool, "replay-frame", rcs, str(k),
                            os.path.join(out, f"{name}_f{k}.cap")], check=True)
        print(f"{name}: {n} frames, {os.path.getsize(rcs)} B")


if __name__ == "__main__":
    main()
