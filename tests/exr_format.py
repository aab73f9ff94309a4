"""Reader for the OpenEXR files the headless host writes (single-part scanline, no
compression), following the public OpenEXR file layout; used by the EXR tests."""
from __future__ import annotations

import struct
from pathlib import Path

import numpy as np


def parse_exr(path: Path) -> tuple[dict, dict]:
    """Returns (header attributes, {channel: (h, w) array}) of a single-part scanline file
    without compression."""
    b = path.read_bytes()
    magic, version = struct.unpack_from("<ii", b, 0)
    assert magic == 20000630 and version == 2
    pos = 8
    attrs = {}

    def cstr(p):
        e = b.index(b"\0", p)
        return b[p:e].decode(), e + 1

    while b[pos] != 0:
        name, pos = cstr(pos)
        typ, pos = cstr(pos)
        (size,) = struct.unpack_from("<i", b, pos)
        pos += 4
        attrs[name] = (typ, b[pos:pos + size])
        pos += size
    pos += 1
    # channel list
    typ, raw = attrs["channels"]
    assert typ == "chlist"
    chans, p = [], 0
    while raw[p] != 0:
        e = raw.index(b"\0", p)
        nm = raw[p:e].decode()
        ptype, _plin, xs, ys = struct.unpack_from("<iB3xii", raw, e + 1)
        assert (xs, ys) == (1, 1)
        chans.append((nm, ptype))
        p = e + 1 + 16
    assert [c for c, _ in chans] == sorted(c for c, _ in chans)
    assert attrs["compression"] == ("compression", b"\x00")
    x0, y0, x1, y1 = struct.unpack("<iiii", attrs["dataWindow"][1])
    assert attrs["displayWindow"] == attrs["dataWindow"] and (x0, y0) == (0, 0)
    assert attrs["lineOrder"] == ("lineOrder", b"\x00")
    assert struct.unpack("<f", attrs["pixelAspectRatio"][1])[0] == 1.0
    assert struct.unpack("<ff", attrs["screenWindowCenter"][1]) == (0.0, 0.0)
    w, h = x1 + 1, y1 + 1
    offsets = struct.unpack_from(f"<{h}Q", b, pos)
    out = {c: np.zeros((h, w), np.float32) for c, _ in chans}
    for y, off in enumerate(offsets):
        ly, size = struct.unpack_from("<ii", b, off)
        assert ly == y
        p = off + 8
        for c, ptype in chans:
            dt = np.float16 if ptype == 1 else np.float32
            n = w * np.dtype(dt).itemsize
            out[c][y] = np.frombuffer(b, dt, count=w, offset=p).astype(np.float32)
            p += n
        assert p - off - 8 == size
    return attrs, out
