"""Reader of uncompressed scanline OpenEXR files (HALF or FLOAT channels).

Reads the reference's init textures (init/*.exr: 1024x512, B/G/R HALF,
no compression) and the thickness frames this library writes.  Written from
the published OpenEXR file layout; other compressions are rejected.
"""
from __future__ import annotations

import struct

import numpy as np


def read_exr(path: str) -> dict:
    """Returns {channel name: float32 array [height, width]}."""
    data = open(path, "rb").read()
    if data[:4] != b"\x76\x2f\x31\x01":
        raise ValueError(f"{path}: not an OpenEXR file")
    flags = struct.unpack_from("<I", data, 4)[0]
    if flags & 0x200 or flags & 0x1000:
        raise ValueError(f"{path}: tiled / multi-part files are not supported")
    pos = 8
    attrs = {}
    while True:
        end = data.index(b"\0", pos)
        name = data[pos:end].decode()
        pos = end + 1
        if not name:
            break
        end = data.index(b"\0", pos)
        typ = data[pos:end].decode()
        pos = end + 1
        size = struct.unpack_from("<i", data, pos)[0]
        pos += 4
        attrs[name] = (typ, data[pos:pos + size])
        pos += size
    if attrs["compression"][1][0] != 0:
        raise ValueError(f"{path}: only uncompressed EXR is supported")
    chans = []
    raw = attrs["channels"][1]
    p = 0
    while raw[p] != 0:
        end = raw.index(b"\0", p)
        cname = raw[p:end].decode()
        ptype = struct.unpack_from("<i", raw, end + 1)[0]
        chans.append((cname, ptype))
        p = end + 1 + 16
    xmin, ymin, xmax, ymax = struct.unpack("<4i", attrs["dataWindow"][1])
    w, h = xmax - xmin + 1, ymax - ymin + 1
    offsets = struct.unpack_from(f"<{h}Q", data, pos)
    out = {c: np.zeros((h, w), dtype=np.float32) for c, _ in chans}
    for off in offsets:
        y, size = struct.unpack_from("<ii", data, off)
        q = off + 8
        for cname, ptype in chans:
            if ptype == 1:
                row = np.frombuffer(data, dtype="<f2", count=w, offset=q).astype(np.float32)
                q += 2 * w
            elif ptype == 2:
                row = np.frombuffer(data, dtype="<f4", count=w, offset=q)
                q += 4 * w
            else:
                raise ValueError("UINT channels are not supported")
            out[cname][y - ymin] = row
    return out
