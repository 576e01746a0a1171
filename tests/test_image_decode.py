"""The image decoders behind recorded streams' images
(rive-runtime_gb300/image_decode.py) and the stream reader's image frames.

The decoders are pinned on known answers built here: PNG rows under every
filter type, a baseline JPEG of DC-only blocks (each block's samples are
128 + DC / 8 with a unit quantiser), and the premultiplication rule of
Bitmap::pixelFormat (decoders/src/bitmap_decoder.cpp:66-89). With the
reference's recordings present, a real frame with images and an image mesh
converts with them."""
import os
import struct
import zlib

import numpy as np
import pytest

from conftest import load_package
import oracle

load_package()
from rive_runtime_gb300 import image_decode, sriv  # noqa: E402


def _png(rgba: np.ndarray, filters) -> bytes:
    """PNG (colour type 6) with row y filtered by filters[y % len]."""
    h, w, _ = rgba.shape
    bpp, stride = 4, w * 4
    rows = rgba.reshape(h, stride).astype(np.int32)
    out = bytearray()
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        ft = filters[y % len(filters)]
        cur = rows[y]
        left = np.concatenate([np.zeros(bpp, np.int32), cur[:-bpp]])
        upleft = np.concatenate([np.zeros(bpp, np.int32), prev[:-bpp]])
        if ft == 0:
            f = cur
        elif ft == 1:
            f = cur - left
        elif ft == 2:
            f = cur - prev
        elif ft == 3:
            f = cur - ((left + prev) >> 1)
        else:
            p = left + prev - upleft
            pa, pb, pc = np.abs(p - left), np.abs(p - prev), np.abs(p - upleft)
            pred = np.where((pa <= pb) & (pa <= pc), left, np.where(pb <= pc, prev, upleft))
            f = cur - pred
        out.append(ft)
        out += (f & 0xFF).astype(np.uint8).tobytes()
        prev = cur

    def chunk(t, d):
        return struct.pack(">I", len(d)) + t + d + struct.pack(">I", zlib.crc32(t + d) & 0xFFFFFFFF)
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0))
            + chunk(b"IDAT", zlib.compress(bytes(out))) + chunk(b"IEND", b""))


def test_png_every_filter_round_trips():
    rng = np.random.default_rng(7)
    img = rng.integers(0, 256, (13, 11, 4), dtype=np.uint8)
    for filters in ([0], [1], [2], [3], [4], [0, 1, 2, 3, 4]):
        assert np.array_equal(image_decode.decode(_png(img, filters)), img), filters


def _jpeg_dc_only(dcs, width, height):
    """A baseline grayscale JPEG whose 8x8 blocks carry only DC terms `dcs`
    (row-major), a unit quantiser, and Huffman tables coding DC categories
    0..11 with 4-bit codes and AC with a lone end-of-block."""
    def seg(marker, body):
        return b"\xff" + bytes([marker]) + struct.pack(">H", len(body) + 2) + body
    dqt = seg(0xDB, b"\x00" + bytes([1] * 64))
    sof = seg(0xC0, struct.pack(">BHHB", 8, height, width, 1) + bytes([1, 0x11, 0]))
    # DC: 12 symbols of length 4 (codes 0000..1011 for categories 0..11).
    dht_dc = seg(0xC4, bytes([0x00]) + bytes([0, 0, 0, 12] + [0] * 12) + bytes(range(12)))
    # AC: one symbol (0x00, end of block) of length 1 (code 0).
    dht_ac = seg(0xC4, bytes([0x10]) + bytes([1] + [0] * 15) + bytes([0]))
    sos = seg(0xDA, bytes([1, 1, 0x00, 0, 63, 0]))
    bits = []
    pred = 0
    for dc in dcs:
        diff = dc - pred
        pred = dc
        s = 0 if diff == 0 else int(abs(diff)).bit_length()
        bits += [int(c) for c in format(s, "04b")]
        if s:
            v = diff if diff > 0 else diff + (1 << s) - 1
            bits += [int(c) for c in format(v, f"0{s}b")]
        bits.append(0)  # end of block
    while len(bits) % 8:
        bits.append(1)
    data = bytearray()
    for i in range(0, len(bits), 8):
        b = int("".join(map(str, bits[i:i + 8])), 2)
        data.append(b)
        if b == 0xFF:
            data.append(0)
    return b"\xff\xd8" + dqt + sof + dht_dc + dht_ac + sos + bytes(data) + b"\xff\xd9"


def test_jpeg_dc_only_blocks_decode_to_their_means():
    dcs = [0, 80, -200, 400, -8, 1016]
    img = image_decode.decode(_jpeg_dc_only(dcs, 24, 16))
    assert img.shape == (16, 24, 4) and (img[..., 3] == 255).all()
    for i, dc in enumerate(dcs):
        by, bx = divmod(i, 3)
        block = img[8 * by:8 * by + 8, 8 * bx:8 * bx + 8, 0]
        want = int(np.clip(np.rint(128 + dc / 8), 0, 255))
        assert (block == want).all(), (i, dc, np.unique(block))
        assert (img[8 * by:8 * by + 8, 8 * bx:8 * bx + 8, 1] == block).all()


def test_premultiply_rounds_to_nearest():
    rng = np.random.default_rng(1)
    rgba = rng.integers(0, 256, (64, 64, 4), dtype=np.uint8)
    got = image_decode.premultiply(rgba)
    want = np.rint(rgba[..., :3].astype(np.float64) * rgba[..., 3:4] / 255.0)
    assert np.array_equal(got[..., :3], want.astype(np.uint8))
    assert np.array_equal(got[..., 3], rgba[..., 3])


SILVERS = os.path.join(oracle.REFERENCE_SOURCES, "tests", "unit_tests", "silvers")


@pytest.mark.skipif(not os.path.isdir(SILVERS), reason="reference recordings absent")
def test_recorded_frame_keeps_its_images_and_mesh():
    with open(os.path.join(SILVERS, "image_fit_alignment_2.sriv"), "rb") as f:
        st = sriv.read_sriv(f.read())
    sc, stats = st.frame_scene(10, images=True)
    assert stats.images == 4 and stats.meshes == 1 and stats.dropped_images == 0
    assert len(sc.meshes) == 1 and len(sc.images) >= 1
    m = sc.meshes[0]
    assert len(m.indices) % 3 == 0 and int(m.indices.max()) < len(m.xy)
    # Without `images` the same frame drops them, as before.
    _, plain = st.frame_scene(10)
    assert plain.dropped_images == 5 and plain.images == 0


def test_malformed_images_are_refused():
    png = _png(np.zeros((4, 4, 4), np.uint8), [0])
    for bad in (png[:40], png[:-20], b"\xff\xd8\xff\xdb\x00", _jpeg_dc_only([5], 8, 8)[:-12],
                b"GIF89a"):
        with pytest.raises(image_decode.DecodeError):
            image_decode.decode(bad)
