"""Test helpers for the EXR initialisers: a small writer of single-part,
scanline, uncompressed OpenEXR files with HALF channels B, G, R (the
layout of the reference's init/*.exr textures), and a numpy restatement of
the bilinear resampling (half-pixel centres, clamped edges) the library
applies to them."""
from __future__ import annotations

import struct

import numpy as np


def write_exr_bgr(path, b, g, r, pixel_type: str = "half") -> None:
    """Write three equally shaped planes as channels B, G, R, HALF (default)
    or FLOAT samples."""
    h, w = b.shape
    code, dt, size = {"half": (1, "<f2", 2), "float": (2, "<f4", 4)}[pixel_type]
    planes = [np.asarray(p, dtype=np.float32).astype(dt) for p in (b, g, r)]
    hdr = bytearray(b"\x76\x2f\x31\x01") + struct.pack("<I", 2)

    def attr(name, typ, data):
        hdr.extend(name.encode() + b"\0" + typ.encode() + b"\0" + struct.pack("<I", len(data)))
        hdr.extend(data)

    ch = b"".join(c.encode() + b"\0" + struct.pack("<iBBBBii", code, 0, 0, 0, 0, 1, 1)
                  for c in ("B", "G", "R")) + b"\0"
    attr("channels", "chlist", ch)
    attr("compression", "compression", b"\0")
    attr("dataWindow", "box2i", struct.pack("<4i", 0, 0, w - 1, h - 1))
    attr("displayWindow", "box2i", struct.pack("<4i", 0, 0, w - 1, h - 1))
    attr("lineOrder", "lineOrder", b"\0")
    attr("pixelAspectRatio", "float", struct.pack("<f", 1.0))
    attr("screenWindowCenter", "v2f", struct.pack("<2f", 0.0, 0.0))
    attr("screenWindowWidth", "float", struct.pack("<f", 1.0))
    hdr.extend(b"\0")
    line = 3 * size * w
    first = len(hdr) + 8 * h
    table = b"".join(struct.pack("<Q", first + (8 + line) * y) for y in range(h))
    body = bytearray()
    for y in range(h):
        body.extend(struct.pack("<iI", y, line))
        for p in planes:
            body.extend(p[y].tobytes())
    with open(path, "wb") as f:
        f.write(bytes(hdr) + table + bytes(body))


def _taps(s: int, dn: int):
    scale = s / dn
    i0 = np.zeros(dn, dtype=np.int64)
    w1 = np.zeros(dn, dtype=np.float32)
    for k in range(dn):
        f = np.float32((k + 0.5) * scale - 0.5)
        i = int(np.floor(f))
        f = np.float32(f - np.float32(i))
        if i < 0:
            i, f = 0, np.float32(0.0)
        if i >= s - 1:
            i, f = s - 1, np.float32(0.0)
        i0[k], w1[k] = i, f
    return i0, w1


def resize_linear(src, dw: int, dh: int) -> np.ndarray:
    """Bilinear resampling in FP32, destination pixel x at source
    (x + 0.5) sw / dw - 0.5, edges clamped (cv::resize INTER_LINEAR)."""
    src = np.asarray(src, dtype=np.float32)
    sh, sw = src.shape
    xi, xw = _taps(sw, dw)
    yi, yw = _taps(sh, dh)
    xj = np.minimum(xi + 1, sw - 1)
    yj = np.minimum(yi + 1, sh - 1)
    one = np.float32(1.0)
    a = xw[None, :]
    r0 = src[yi]
    r1 = src[yj]
    top = r0[:, xi] * (one - a) + r0[:, xj] * a
    bot = r1[:, xi] * (one - a) + r1[:, xj] * a
    b = yw[:, None]
    return (top * (one - b) + bot * b).astype(np.float32)
