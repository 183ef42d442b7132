"""The gpro GeoTIFF codec (pargo_gb300/gpro/src/geotiff.cpp).  The reader on
the TIFF forms it accepts -- classic TIFF and BigTIFF, either byte order;
strips of one row, several rows or the whole image; tiles with ragged right
and bottom edges; 8/16/32/64-bit unsigned and signed integers and 32/64-bit
floats -- against the values the file holds, read through a C++ driver
(tests/cpp/tiff_dump.cpp); the georeferencing and nodata tags; the refusal of
compressed, truncated and malformed files.  The writer's BigTIFF form, read
back by the same reader and checked field by field."""
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
               compression=1, truncate=0, bigtiff=False):
    """A TIFF of `arr` in the given byte order, classic or BigTIFF; layout
    ("strips", k) (k rows per strip, 0 = all) or ("tiles", tw, tl)."""
    bo = ">" if big else "<"
    osz, ofmt, otype = (8, "Q", 16) if bigtiff else (4, "I", 4)   # offsets and byte counts: LONG8 or LONG
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
    add(off_tag, otype, [0] * len(chunks))
    add(cnt_tag, otype, [len(c) for c in chunks])
    entries.sort(key=lambda e: e[0])
    inline = 8 if bigtiff else 4
    head = 16 if bigtiff else 8
    ifd_size = 8 + 20 * len(entries) + 8 if bigtiff else 2 + 12 * len(entries) + 4
    cursor = head + ifd_size
    value_off = {}
    for i, (tag, typ, count, payload) in enumerate(entries):
        if len(payload) > inline:
            value_off[i] = cursor
            cursor += len(payload) + (len(payload) & 1)
    chunk_off = []
    for c in chunks:
        chunk_off.append(cursor)
        cursor += len(c)
    for i, e in enumerate(entries):
        if e[0] == off_tag:
            entries[i] = (e[0], e[1], e[2], struct.pack(bo + ofmt * len(chunk_off), *chunk_off))
    out = bytearray(b"MM" if big else b"II")
    if bigtiff:
        out += struct.pack(bo + "HHHQ", 43, 8, 0, head) + struct.pack(bo + "Q", len(entries))
    else:
        out += struct.pack(bo + "HI", 42, head) + struct.pack(bo + "H", len(entries))
    for i, (tag, typ, count, payload) in enumerate(entries):
        out += struct.pack(bo + ("HHQ" if bigtiff else "HHI"), tag, typ, count)
        if len(payload) > inline:
            out += struct.pack(bo + ofmt, value_off[i])
        else:
            out += payload.ljust(inline, b"\0")
    out += struct.pack(bo + ofmt, 0)
    for i, (tag, typ, count, payload) in enumerate(entries):
        if len(payload) > inline:
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
@pytest.mark.parametrize("layout,bigtiff", [(("strips", 1), False), (("strips", 7), False), (("strips", 0), False),
                                            (("tiles", 16, 16), False), (("strips", 7), True),
                                            (("tiles", 16, 16), True)])
def test_reader_sample_types_byte_orders_and_layouts(bits, fmt, kind, big, layout, bigtiff, dump_exe, tmp_path):
    arr = _values(kind, (37, 45), bits * 7 + fmt)
    path = tmp_path / "in.tif"
    build_tiff(path, arr, bits, fmt, big, layout, bigtiff=bigtiff)
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


def _bigtiff_fields(path):
    """Header and first IFD of a little-endian BigTIFF: {tag: (type, count, value bytes)}."""
    b = open(path, "rb").read()
    assert b[:2] == b"II" and struct.unpack("<HHH", b[2:8]) == (43, 8, 0)
    ifd = struct.unpack("<Q", b[8:16])[0]
    n = struct.unpack("<Q", b[ifd:ifd + 8])[0]
    out = {}
    for i in range(n):
        e = ifd + 8 + 20 * i
        tag, typ, count = struct.unpack("<HHQ", b[e:e + 12])
        size = {2: 1, 3: 2, 4: 4, 12: 8, 16: 8}[typ] * count
        off = e + 12 if size <= 8 else struct.unpack("<Q", b[e + 12:e + 20])[0]
        out[tag] = (typ, count, b[off:off + size])
    return out, b


@pytest.mark.parametrize("dtype,shape", [(0, (37, 45)), (1, (37, 45)), (0, (3, 20000)), (1, (1, 1))])
def test_writer_bigtiff_form(dtype, shape, dump_exe, tmp_path):
    """write_geotiff's BigTIFF output (chosen on its own above 4 GB, asked for
    here on small rasters): LONG8 strip offsets and byte counts that locate
    the samples, and the reader's values, tags and transform equal to what
    was written -- the same as the classic file of the same raster."""
    rows, cols = shape
    expect = (np.arange(rows * cols, dtype=np.float64) - 7.25).reshape(rows, cols)
    if dtype == 0:
        expect = expect.astype(np.float32).astype(np.float64)
    paths = {}
    for big in (0, 1):
        paths[big] = tmp_path / ("w%d.tif" % big)
        r = subprocess.run([dump_exe, "--write", str(paths[big]), str(rows), str(cols), str(dtype), str(big)],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stdout
    fields, raw = _bigtiff_fields(paths[1])
    assert fields[256][2] == struct.pack("<I", cols) and fields[257][2] == struct.pack("<I", rows)
    offs_t, noffs, offs = fields[273]
    cnts_t, ncnts, cnts = fields[279]
    assert offs_t == 16 and cnts_t == 16 and noffs == ncnts
    offs = struct.unpack("<%dQ" % noffs, offs)
    cnts = struct.unpack("<%dQ" % ncnts, cnts)
    data = b"".join(raw[o:o + c] for o, c in zip(offs, cnts))
    got = np.frombuffer(data, dtype="<f4" if dtype == 0 else "<f8").astype(np.float64).reshape(rows, cols)
    assert np.array_equal(got, expect)
    reads = [read_with_gpro(dump_exe, paths[big], tmp_path)[0] for big in (0, 1)]
    for rd in reads:
        assert rd is not None
        assert np.array_equal(rd["values"], expect)
        assert rd["dtype"] == dtype and rd["has_nodata"] and rd["nodata"] == -9999.0
        assert rd["transform"] == (500.0, 30.0, 0.0, 9000.0, 0.0, -30.0)
    assert open(paths[0], "rb").read(4) == b"II*\0"


def test_reader_refuses_malformed_headers(dump_exe, tmp_path):
    p = tmp_path / "m.tif"
    arr = _values("f4", (10, 12), 3)
    build_tiff(p, arr, 32, 3, False, ("strips", 4))
    good = bytearray(p.read_bytes())
    bad = bytearray(good)
    bad[2:4] = struct.pack("<H", 44)                      # neither classic TIFF nor BigTIFF
    p.write_bytes(bytes(bad))
    got, err = read_with_gpro(dump_exe, p, tmp_path)
    assert got is None and "BigTIFF" in err
    bad = bytearray(good)
    bad[4:8] = struct.pack("<I", len(good) + 100)         # first IFD past the end
    p.write_bytes(bytes(bad))
    got, err = read_with_gpro(dump_exe, p, tmp_path)
    assert got is None and "truncated" in err
    build_tiff(p, np.zeros((0, 5), np.float32), 32, 3, False, ("strips", 1))   # an empty image
    got, err = read_with_gpro(dump_exe, p, tmp_path)
    assert got is None
