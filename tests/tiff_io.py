"""Minimal GeoTIFF reading/writing for the tests (uncompressed strips,
float32/float64, little- or big-endian input; little-endian output)."""
import struct

import numpy as np


def read_tiff(path):
    """(array, nodata, cellsize) of a single-band uncompressed strip TIFF."""
    b = open(path, "rb").read()
    bo = "<" if b[:2] == b"II" else ">"
    off = struct.unpack(bo + "I", b[4:8])[0]
    n = struct.unpack(bo + "H", b[off:off + 2])[0]
    sizes = {1: 1, 2: 1, 3: 2, 4: 4, 11: 4, 12: 8}
    fmts = {1: "B", 2: "c", 3: "H", 4: "I", 11: "f", 12: "d"}
    tags = {}
    for i in range(n):
        e = b[off + 2 + 12 * i: off + 14 + 12 * i]
        tag, typ, cnt = struct.unpack(bo + "HHI", e[:8])
        sz = sizes[typ] * cnt
        raw = e[8:8 + sz] if sz <= 4 else b[struct.unpack(bo + "I", e[8:12])[0]:][:sz]
        tags[tag] = raw.decode().rstrip("\0 ") if typ == 2 else struct.unpack(bo + fmts[typ] * cnt, raw)
    cols, rows, bits = tags[256][0], tags[257][0], tags[258][0]
    fmt = tags.get(339, (1,))[0]
    assert tags[259][0] == 1 and fmt == 3 and bits in (32, 64), "float32/float64 uncompressed only"
    dt = np.dtype(bo + ("f4" if bits == 32 else "f8"))
    data = b"".join(b[o:o + c] for o, c in zip(tags[273], tags[279]))
    arr = np.frombuffer(data, dtype=dt, count=rows * cols).reshape(rows, cols)
    arr = arr.astype(np.float32 if bits == 32 else np.float64)
    nodata = float(tags[42113]) if 42113 in tags else None
    cellsize = tags[33550][0] if 33550 in tags else 1.0
    return arr, nodata, cellsize


def write_tiff(path, arr, nodata, cellsize, origin=(0.0, 0.0)):
    """Single-strip GeoTIFF with pixel scale, tiepoint and GDAL_NODATA: float64
    for a float64 array, float32 otherwise."""
    f64 = np.asarray(arr).dtype == np.float64
    a = np.ascontiguousarray(arr, np.float64 if f64 else np.float32)
    rows, cols = a.shape
    nd = ("%.17g" % nodata).encode() + b"\0"
    entries = []  # (tag, type, count, payload bytes)

    def add(tag, typ, count, payload):
        entries.append((tag, typ, count, payload))
    add(256, 4, 1, struct.pack("<I", cols))
    add(257, 4, 1, struct.pack("<I", rows))
    add(258, 3, 1, struct.pack("<H", 64 if f64 else 32))
    add(259, 3, 1, struct.pack("<H", 1))
    add(262, 3, 1, struct.pack("<H", 1))
    add(273, 4, 1, b"\0\0\0\0")
    add(277, 3, 1, struct.pack("<H", 1))
    add(278, 4, 1, struct.pack("<I", rows))
    add(279, 4, 1, struct.pack("<I", a.nbytes))
    add(339, 3, 1, struct.pack("<H", 3))
    add(33550, 12, 3, struct.pack("<3d", cellsize, cellsize, 0.0))
    add(33922, 12, 6, struct.pack("<6d", 0, 0, 0, origin[0], origin[1], 0))
    add(42113, 2, len(nd), nd)
    ifd_size = 2 + 12 * len(entries) + 4
    cursor = 8 + ifd_size
    extra = b""
    offs = []
    for tag, typ, count, payload in entries:
        if len(payload) > 4:
            offs.append(cursor + len(extra))
            extra += payload + (b"\0" if len(payload) % 2 else b"")
        else:
            offs.append(None)
    data_off = 8 + ifd_size + len(extra)
    out = b"II" + struct.pack("<HI", 42, 8) + struct.pack("<H", len(entries))
    for (tag, typ, count, payload), o in zip(entries, offs):
        if tag == 273:
            payload = struct.pack("<I", data_off)
        out += struct.pack("<HHI", tag, typ, count)
        out += struct.pack("<I", o) if o is not None else payload.ljust(4, b"\0")
    out += struct.pack("<I", 0) + extra + a.astype("<f8" if f64 else "<f4").tobytes()
    with open(path, "wb") as fh:
        fh.write(out)
