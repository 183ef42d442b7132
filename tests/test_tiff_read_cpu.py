"""The gpro GeoTIFF reader (pargo_gb300/gpro/src/geotiff.cpp) on the TIFF
forms it accepts -- either byte order; strips of one row, several rows or the
whole image; tiles with ragged right and bottom edges; 8/16/32/64-bit
unsigned and signed integers and 32/64-bit floats -- against the values the
file holds, read through a C++ driver (tests/cpp/tiff_dump.cpp).  Also the
georeferencing and nodata tags, and the refusal of compressed or truncated
files."""
import os
import struct
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from pargo_gb300 import _paths

INC = [os.path.join(ROOT, "pargo_gb300", "gpro", "include"), os.path.join(ROOT, "include")]


@pytest.fixture(scope="module")
def dump_exe(tmp_path_factory):
    exe = tmp_path_factory.mktemp("tiffdump") / "tiff_dump"
    cmd = ["g++", "-std=c++14", "-O1", "-Wall"] + ["-I" + d for d in INC] + \
          [os.path.join(ROOT, "tests", "cpp", "tiff_dump.cpp"), "-o", str(exe),
           "-L" + _paths.LIB_DIR, "-lpargo_gpro", "-lpargo_gpu", "-Wl,-rpath," + _paths.LIB_DIR]
    subprocess.run(cmd, check=True)
    return str(exe)


def read_with_gpro(exe, path, tmp_path):
    out = tmp_path / "dump.bin"
    r = subprocess.run([exe, str(path), str(out)], capture_output=True, text=True)
    if r.returncode != 0:
        return None, r.stdout.strip()
    b = out.read_bytes()
    rows, cols, dtype, has_nd = struct.unpack("<4q", b[:32])
    nodata = struct.unpack("<d", b[32:40])[0]
    transform = struct.unpack("<6d", b[40:88])
    values = np.frombuffer(b[88:], dtype="<f8").reshape(rows, cols)
    return dict(dtype=dtype, has_nodata=bool(has_nd), nodata=nodata, transform=transform, values=values), ""


# (bits, SampleFormat, numpy kind): 1 unsigned, 2 signed, 3 IEEE float
SAMPLE_TYPES = [(8, 1, "u1"), (8, 2, "i1"), (16, 1, "u2"), (16, 2, "i2"), (32, 1, "u4"), (32, 2, "i4"),
                (64, 2, "i8"), (32, 3, "f4"), (64, 3, "f8")]


def build_tiff(path, arr, bits, fmt, big, layout, nodata="-9999", scale=(30.0, 30.0), tie=(500.0, 9000.0),
               compression=1, truncate=0):
    """A classic TIFF of `arr` in the given byte order; layout ("strips", k)
    (k rows per strip, 0 = all) or ("tiles", tw, tl)."""
    bo = ">" if big else "<"
    rows, cols = arr.shape
    data = np.ascontiguousarray(arr).astype(bo + np.dtype(arr.dtype).str[1:])
    entries = []   # (tag, type, count, payload bytes)

    def add(tag, typ, values):
        fmtc = {3: "H", 4: "I", 12: "d", 2: "s", 16: "Q"}[typ]
        if typ == 2:
            payload = values.encode() + b"\0"
            count = len(payload)
        else:
            payload = struct.pack(bo + fmtc * len(values), *values)
            count = len(values)
        entries.append((tag, typ, count, payload))

    add(256, 4, [cols])
    add(257, 4, [rows])
    add(258, 3, [bits])
    add(259, 3, [compression])
    add(262, 3, [1])
    add(277, 3, [1])
    add(339, 3, [fmt])
    add(33550, 12, [scale[0], scale[1], 0.0])
    add(33922, 12, [0.0, 0.0, 0.0, tie[0], tie[1], 0.0])
    if nodata is not None:
        add(42113, 2, nodata)
    bpp = bits // 8
    chunks = []
    if layout[0] == "strips":
        per = layout[1] or rows
        for r0 in range(0, rows, per):
            chunks.append(data[r0:r0 + per].tobytes())
        add(278, 4, [per])
    else:
        tw, tl = layout[1], layout[2]
        for ty in range(0, rows, tl):
            for tx in range(0, cols, tw):
                t = np.zeros((tl, tw), dtype=data.dtype)
                blk = data[ty:ty + tl, tx:tx + tw]
                t[:blk.shape[0], :blk.shape[1]] = blk
                chunks.append(t.tobytes())
        add(322, 4, [tw])
        add(323, 4, [tl])
    # offsets are patched once the layout is known
    off_tag, cnt_tag = (273, 279) if layout[0] == "strips" else (324, 325)
    add(off_tag, 4, [0] * len(chunks))
    add(cnt_tag, 4, [len(c) for c in chunks])
    entries.sort(key=lambda e: e[0])
    ifd_size = 2 + 12 * len(entries) + 4
    cursor = 8 + ifd_size
    value_off = {}
    for i, (tag, typ, count, payload) in enumerate(entries):
        if len(payload) > 4:
            value_off[i] = cursor
            cursor += len(payload) + (len(payload) & 1)
    chunk_off = []
    for c in chunks:
        chunk_off.append(cursor)
        cursor += len(c)
    for i, e in enumerate(entries):
        if e[0] == off_tag:
            entries[i] = (e[0], e[1], e[2], struct.pack(bo + "I" * len(chunk_off), *chunk_off))
    out = bytearray(b"MM\0*" if big else b"II*\0")
    out += struct.pack(bo + "I", 8)
    out += struct.pack(bo + "H", len(entries))
    for i, (tag, typ, count, payload) in enumerate(entries):
        out += struct.pack(bo + "HHI", tag, typ, count)
        out += struct.pack(bo + "I", value_off[i]) if len(payload) > 4 else payload.ljust(4, b"\0")
    out += struct.pack(bo + "I", 0)
    for i, (tag, typ, count, payload) in enumerate(entries):
        if len(payload) > 4:
            out += payload + (b"\0" if len(payload) & 1 else b"")
    for c in chunks:
        out += c
    if truncate:
        out = out[:-truncate]
    with open(path, "wb") as f:
        f.write(bytes(out))


def _values(kind, shape, seed):
    rng = np.random.default_rng(seed)
    dt = np.dtype(kind)
    if dt.kind == "f":
        v = (rng.standard_normal(shape) * 1000).astype(dt)
        v.flat[::17] = -9999.0
        return v
    info = np.iinfo(dt)
    lo, hi = max(info.min, -(2 ** 40)), min(info.max, 2 ** 40)
    return rng.integers(lo, hi, size=shape, endpoint=True, dtype=np.int64).astype(dt)


@pytest.mark.parametrize("bits,fmt,kind", SAMPLE_TYPES)
@pytest.mark.parametrize("big", [False, True])
@pytest.mark.parametrize("layout", [("strips", 1), ("strips", 7), ("strips", 0), ("tiles", 16, 16)])
def test_reader_sample_types_byte_orders_and_layouts(bits, fmt, kind, big, layout, dump_exe, tmp_path):
    arr = _values(kind, (37, 45), bits * 7 + fmt)
    path = tmp_path / "in.tif"
    build_tiff(path, arr, bits, fmt, big, layout)
    got, err = read_with_gpro(dump_exe, path, tmp_path)
    assert got is not None, err
    assert np.array_equal(got["values"], arr.astype(np.float64))
    want_dtype = {(32, 3): 0, (64, 3): 1}.get((bits, fmt), {8: 2, 16: 3}.get(bits, 4))  # pargo_dtype
    assert got["dtype"] == want_dtype
    assert got["has_nodata"] and got["nodata"] == -9999.0
    assert got["transform"] == (500.0, 30.0, 0.0, 9000.0, 0.0, -30.0)


def test_reader_refuses_compressed_and_truncated_files(dump_exe, tmp_path):
    arr = _values("f4", (20, 30), 1)
    p = tmp_path / "c.tif"
    build_tiff(p, arr, 32, 3, False, ("strips", 4), compression=5)
    got, err = read_with_gpro(dump_exe, p, tmp_path)
    assert got is None and "uncompressed" in err
    for layout in (("strips", 4), ("tiles", 16, 16)):
        build_tiff(p, arr, 32, 3, False, layout, truncate=10)
        got, err = read_with_gpro(dump_exe, p, tmp_path)
        assert got is None and "truncated" in err, err
    p.write_bytes(b"not a tiff at all")
    got, err = read_with_gpro(dump_exe, p, tmp_path)
    assert got is None and "not a TIFF" in err
