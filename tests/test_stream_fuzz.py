"""Malformed input to the call-stream readers: random byte flips and
truncations of valid streams either read or raise the reader's own error
(SrivError, CmdbufError), never another exception, and finish promptly."""
import os

import numpy as np

from conftest import load_package

load_package()
from rive_runtime_gb300 import cmdbuf, sriv  # noqa: E402

from test_sriv import _two_frame_stream  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def _mutations(data: bytes, rng, count):
    for _ in range(count):
        b = bytearray(data)
        kind = rng.integers(3)
        if kind == 0:
            for _ in range(rng.integers(1, 6)):
                b[rng.integers(len(b))] = int(rng.integers(256))
        elif kind == 1:
            b = b[:rng.integers(len(b))]
        else:
            i = rng.integers(len(b))
            b[i:i] = bytes(rng.integers(0, 256, rng.integers(1, 9)).astype(np.uint8))
        yield bytes(b)


def test_sriv_reader_survives_corruption():
    rng = np.random.default_rng(5)
    base = _two_frame_stream()
    for data in _mutations(base, rng, 2000):
        try:
            st = sriv.read_sriv(data, default_size=(32, 32))
            for k in range(len(st.frames)):
                st.frame_scene(k)[0].to_bytes()
        except sriv.SrivError:
            pass


def test_command_stream_reader_survives_corruption():
    rng = np.random.default_rng(6)
    with open(os.path.join(HERE, "golden", "cmdbuf", "component_list_grouped.rcs"), "rb") as f:
        frames, hdr = cmdbuf.read_rcs(f.read())
    commands, blobs = frames[0]
    for i, data in enumerate(_mutations(commands, rng, 300)):
        try:
            cmdbuf.command_buffer_scene(data, blobs, **hdr)[0].to_bytes()
        except cmdbuf.CmdbufError:
            pass
    for data in _mutations(blobs, rng, 100):
        try:
            cmdbuf.command_buffer_scene(commands, data, **hdr)[0].to_bytes()
        except cmdbuf.CmdbufError:
            pass
