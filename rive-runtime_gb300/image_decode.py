"""Decoders for the encoded images recorded streams carry (the bytes a
SerializingFactory writes for Factory::decodeImage,
utils/serializing_factory.cpp:466-480): PNG (ISO/IEC 15948) with 8-bit
samples, not interlaced, and baseline sequential JPEG (ITU-T T.81, Huffman,
8-bit). They turn a recorded frame's images into the RGBA8 texels a scene
recording hands RenderContextImpl::makeImageTexture.

`decode(data)` returns (height, width, 4) uint8 straight RGBA;
`premultiply(rgba)` applies Bitmap::pixelFormat(RGBAPremul)
(decoders/src/bitmap_decoder.cpp:36-99): each colour channel times alpha,
divided by 255 rounded to nearest (simd::div255), alpha kept. The JPEG path
uses a floating-point inverse DCT and replicates chroma samples: any decoder
may differ from another in the last bit of a sample, and nothing here depends
on which, since the texels travel with the recording.
"""
from __future__ import annotations

import struct
import zlib

import numpy as np


class DecodeError(ValueError):
    pass


def decode(data: bytes) -> np.ndarray:
    """Straight RGBA8 (height, width, 4); DecodeError for anything malformed,
    truncated or in a form not handled here."""
    try:
        if data[:8] == b"\x89PNG\r\n\x1a\n":
            return decode_png(data)
        if data[:2] == b"\xff\xd8":
            return decode_jpeg(data)
    except DecodeError:
        raise
    except (ValueError, KeyError, IndexError, struct.error, zlib.error) as e:
        raise DecodeError(f"malformed image: {e}") from e
    raise DecodeError("neither a PNG nor a JPEG")


def premultiply(rgba: np.ndarray) -> np.ndarray:
    a = rgba[..., 3:4].astype(np.uint32)
    x = rgba[..., :3].astype(np.uint32) * a + 128
    rgb = (x + (x >> 8)) >> 8
    return np.concatenate([rgb.astype(np.uint8), rgba[..., 3:4]], -1)


# ---- PNG ---------------------------------------------------------------------

def _paeth(a, b, c):
    p = a + b - c
    pa, pb, pc = abs(p - a), abs(p - b), abs(p - c)
    if pa <= pb and pa <= pc:
        return a
    return b if pb <= pc else c


def _unfilter(raw: bytes, height: int, stride: int, bpp: int) -> np.ndarray:
    out = np.zeros((height, stride), np.uint8)
    prev = np.zeros(stride, np.int32)
    pos = 0
    for y in range(height):
        ft = raw[pos]
        line = np.frombuffer(raw, np.uint8, stride, pos + 1).astype(np.int32)
        pos += stride + 1
        if ft == 0:
            cur = line
        elif ft == 2:  # up
            cur = (line + prev) & 0xFF
        elif ft in (1, 3, 4):
            # Sub, Average and Paeth depend on the bytes to the left: walk
            # the row in steps of one pixel.
            cur = line.copy()
            for x in range(stride):
                left = int(cur[x - bpp]) if x >= bpp else 0
                up = int(prev[x])
                if ft == 1:
                    pred = left
                elif ft == 3:
                    pred = (left + up) >> 1
                else:
                    pred = _paeth(left, up, int(prev[x - bpp]) if x >= bpp else 0)
                cur[x] = (cur[x] + pred) & 0xFF
        else:
            raise DecodeError(f"bad PNG filter {ft}")
        out[y] = cur
        prev = cur
    return out


def decode_png(data: bytes) -> np.ndarray:
    pos = 8
    idat = []
    width = height = depth = ctype = interlace = None
    palette = trns = None
    while pos + 8 <= len(data):
        n, kind = struct.unpack_from(">I4s", data, pos)
        body = data[pos + 8:pos + 8 + n]
        pos += 12 + n
        if kind == b"IHDR":
            width, height, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
        elif kind == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = body
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if width is None or not idat:
        raise DecodeError("PNG without IHDR or IDAT")
    if depth != 8 or interlace != 0:
        raise DecodeError(f"PNG depth {depth} / interlace {interlace} not handled")
    channels = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}.get(ctype)
    if channels is None:
        raise DecodeError(f"PNG colour type {ctype}")
    raw = zlib.decompress(b"".join(idat))
    px = _unfilter(raw, height, width * channels, channels).reshape(height, width, channels)
    out = np.empty((height, width, 4), np.uint8)
    if ctype == 0:
        out[..., :3] = px
        out[..., 3] = 255
        if trns is not None and len(trns) >= 2:
            out[..., 3][px[..., 0] == struct.unpack(">H", trns[:2])[0]] = 0
    elif ctype == 2:
        out[..., :3] = px
        out[..., 3] = 255
        if trns is not None and len(trns) >= 6:
            key = np.array(struct.unpack(">3H", trns[:6]), np.int32)
            out[..., 3][(px.astype(np.int32) == key).all(-1)] = 0
    elif ctype == 3:
        if palette is None:
            raise DecodeError("indexed PNG without a palette")
        alpha = np.full(256, 255, np.uint8)
        if trns is not None:
            alpha[:len(trns)] = np.frombuffer(trns, np.uint8)
        idx = px[..., 0]
        pal = np.zeros((256, 3), np.uint8)
        pal[:len(palette)] = palette
        out[..., :3] = pal[idx]
        out[..., 3] = alpha[idx]
    elif ctype == 4:
        out[..., :3] = px[..., :1]
        out[..., 3] = px[..., 1]
    else:
        out[:] = px
    return out


# ---- Baseline JPEG -------------------------------------------------------------

_ZIGZAG = np.array([
    0, 1, 8, 16, 9, 2, 3, 10, 17, 24, 32, 25, 18, 11, 4, 5,
    12, 19, 26, 33, 40, 48, 41, 34, 27, 20, 13, 6, 7, 14, 21, 28,
    35, 42, 49, 56, 57, 50, 43, 36, 29, 22, 15, 23, 30, 37, 44, 51,
    58, 59, 52, 45, 38, 31, 39, 46, 53, 60, 61, 54, 47, 55, 62, 63], np.int64)


def _idct_matrix():
    # Orthonormal DCT-II basis: X = C x C^T, so x = C^T X C.
    k = np.arange(8)
    c = np.cos((2 * k[None, :] + 1) * k[:, None] * np.pi / 16) * 0.5
    c[0] *= 1 / np.sqrt(2)
    return c


_IDCT = _idct_matrix()


class _Bits:
    """Entropy-coded segment reader: byte stuffing removed, markers stop it."""

    def __init__(self, data: bytes, pos: int):
        self.d = data
        self.p = pos
        self.acc = 0
        self.n = 0
        self.marker = None

    def _fill(self):
        while self.n <= 24:
            b = 0
            if self.marker is None and self.p < len(self.d):
                b = self.d[self.p]
                if b == 0xFF:
                    nxt = self.d[self.p + 1] if self.p + 1 < len(self.d) else 0
                    if nxt == 0x00:
                        self.p += 2
                    else:
                        self.marker = nxt  # stop before the marker; feed zeros
                        b = 0
                else:
                    self.p += 1
            # Keep only the bits not yet consumed.
            self.acc = ((self.acc << 8) | b) & ((1 << (self.n + 8)) - 1)
            self.n += 8

    def bits(self, k: int) -> int:
        if k == 0:
            return 0
        if self.n < k:
            self._fill()
        self.n -= k
        return (self.acc >> self.n) & ((1 << k) - 1)

    def reset(self):
        """At a restart marker: drop the partial byte and the marker."""
        self.acc = self.n = 0
        if self.marker is not None:
            self.p += 2
            self.marker = None


class _Huffman:
    def __init__(self, counts, symbols):
        # Canonical codes: per length, the first code and the symbols.
        self.maxcode = [-1] * 17
        self.valptr = [0] * 17
        self.mincode = [0] * 17
        self.symbols = symbols
        code = k = 0
        for length in range(1, 17):
            n = counts[length - 1]
            if n:
                self.valptr[length] = k
                self.mincode[length] = code
                code += n
                k += n
                self.maxcode[length] = code - 1
            code <<= 1

    def decode(self, bits: _Bits) -> int:
        code = 0
        for length in range(1, 17):
            code = (code << 1) | bits.bits(1)
            if code <= self.maxcode[length]:
                return self.symbols[self.valptr[length] + code - self.mincode[length]]
        raise DecodeError("bad Huffman code")


def _extend(v: int, s: int) -> int:
    return v - (1 << s) + 1 if s and v < (1 << (s - 1)) else v


def decode_jpeg(data: bytes) -> np.ndarray:
    pos = 2
    qt = {}
    hts = {}
    comps = []
    width = height = 0
    restart = 0
    planes = None
    while pos < len(data):
        if data[pos] != 0xFF:
            raise DecodeError("JPEG marker expected")
        m = data[pos + 1]
        pos += 2
        if m == 0xD8 or 0xD0 <= m <= 0xD7:
            continue
        if m == 0xD9:
            break
        (n,) = struct.unpack_from(">H", data, pos)
        seg = data[pos + 2:pos + n]
        pos += n
        if m == 0xDB:
            i = 0
            while i < len(seg):
                pq, tq = seg[i] >> 4, seg[i] & 15
                if pq:
                    qt[tq] = np.array(struct.unpack_from(">64H", seg, i + 1), np.float64)
                    i += 129
                else:
                    qt[tq] = np.frombuffer(seg, np.uint8, 64, i + 1).astype(np.float64)
                    i += 65
        elif m == 0xC4:
            i = 0
            while i < len(seg):
                tc, th = seg[i] >> 4, seg[i] & 15
                counts = list(seg[i + 1:i + 17])
                total = sum(counts)
                hts[(tc, th)] = _Huffman(counts, list(seg[i + 17:i + 17 + total]))
                i += 17 + total
        elif m == 0xC0 or m == 0xC1:
            if seg[0] != 8:
                raise DecodeError("JPEG sample precision other than 8")
            height, width = struct.unpack_from(">HH", seg, 1)
            for k in range(seg[5]):
                cid, hv, tq = seg[6 + 3 * k:9 + 3 * k]
                comps.append({"id": cid, "h": hv >> 4, "v": hv & 15, "tq": tq})
        elif 0xC2 <= m <= 0xCF and m not in (0xC4, 0xC8, 0xCC):
            raise DecodeError(f"JPEG frame type {m:#x} (only baseline) not handled")
        elif m == 0xDD:
            (restart,) = struct.unpack_from(">H", seg, 0)
        elif m == 0xDA:
            planes, pos = _scan(data, pos, seg, comps, qt, hts, width, height, restart)
    if planes is None:
        raise DecodeError("JPEG without a scan")
    return _to_rgba(planes, comps, width, height)


def _scan(data, pos, seg, comps, qt, hts, width, height, restart):
    ns = seg[0]
    byid = {c["id"]: c for c in comps}
    order = []
    for k in range(ns):
        c = byid[seg[1 + 2 * k]]
        c["td"], c["ta"] = seg[2 + 2 * k] >> 4, seg[2 + 2 * k] & 15
        order.append(c)
    if ns != len(comps):
        raise DecodeError("non-interleaved JPEG scans not handled")
    hmax = max(c["h"] for c in comps)
    vmax = max(c["v"] for c in comps)
    mcux = (width + 8 * hmax - 1) // (8 * hmax)
    mcuy = (height + 8 * vmax - 1) // (8 * vmax)
    coefs = {c["id"]: np.zeros((mcuy * c["v"], mcux * c["h"], 64), np.float64) for c in comps}
    pred = {c["id"]: 0 for c in comps}
    bits = _Bits(data, pos)
    left = restart
    for my in range(mcuy):
        for mx in range(mcux):
            if restart:
                if left == 0:
                    bits.reset()
                    for c in comps:
                        pred[c["id"]] = 0
                    left = restart
                left -= 1
            for c in order:
                dc, ac = hts[(0, c["td"])], hts[(1, c["ta"])]
                for by in range(c["v"]):
                    for bx in range(c["h"]):
                        blk = coefs[c["id"]][my * c["v"] + by, mx * c["h"] + bx]
                        s = dc.decode(bits)
                        pred[c["id"]] += _extend(bits.bits(s), s)
                        blk[0] = pred[c["id"]]
                        k = 1
                        while k < 64:
                            rs = ac.decode(bits)
                            r, s = rs >> 4, rs & 15
                            if s == 0:
                                if r != 15:
                                    break
                                k += 16
                                continue
                            k += r
                            if k > 63:
                                raise DecodeError("JPEG coefficient index past 63")
                            blk[k] = _extend(bits.bits(s), s)
                            k += 1
    # The scan ends at the next marker.
    end = bits.p
    while end + 1 < len(data) and not (data[end] == 0xFF and data[end + 1] not in (0, *range(0xD0, 0xD8))):
        end += 1
    planes = {}
    for c in comps:
        q = qt[c["tq"]]
        co = coefs[c["id"]] * q  # dequantised, in zigzag order
        nat = np.zeros_like(co)
        nat[..., _ZIGZAG] = co
        blocks = nat.reshape(co.shape[0], co.shape[1], 8, 8)
        px = np.einsum("ki,abkl,lj->abij", _IDCT, blocks, _IDCT) + 128.0
        plane = px.transpose(0, 2, 1, 3).reshape(co.shape[0] * 8, co.shape[1] * 8)
        planes[c["id"]] = plane
    return planes, end


def _to_rgba(planes, comps, width, height):
    hmax = max(c["h"] for c in comps)
    vmax = max(c["v"] for c in comps)
    full = []
    for c in comps:
        p = planes[c["id"]]
        p = np.repeat(np.repeat(p, vmax // c["v"], 0), hmax // c["h"], 1)
        full.append(p[:height, :width])
    out = np.empty((height, width, 4), np.uint8)
    out[..., 3] = 255
    if len(full) == 1:
        g = np.clip(np.rint(full[0]), 0, 255).astype(np.uint8)
        out[..., 0] = out[..., 1] = out[..., 2] = g
        return out
    if len(full) != 3:
        raise DecodeError(f"JPEG with {len(full)} components not handled")
    y, cb, cr = full[0], full[1] - 128.0, full[2] - 128.0
    # JFIF colour conversion.
    r = y + 1.402 * cr
    g = y - 0.344136 * cb - 0.714136 * cr
    b = y + 1.772 * cb
    for i, ch in enumerate((r, g, b)):
        out[..., i] = np.clip(np.rint(ch), 0, 255).astype(np.uint8)
    return out
