"""Generate the golden fixtures in tests/golden/ from the REFERENCE operators.

Run where the PaRGO reference tree exists (it builds oracle/_ref/ from it):

    python tests/golden/make_golden.py [--reference-root /path/to/PaRGO]

For every case the script records the input DEM and what the unmodified
reference operators (compiled by oracle/build.py, driven by
oracle/ref_driver.cpp) output for it:

  slope_m{0..6}   SlopeOperator, methods FD FFD MD SD SFD TFD TFDW
  d8_8, d8_256    D8Operator on the DEM, dirType 8 and 256
  fill, fill_sweeps   PitRemoveOperator output and its Work() sweep count
  d8w_8           D8Operator on the (float64) pit-removed surface
  sca_conv        SCAOperator on d8w_8 iterated to convergence
  sca_ship        SCAOperator on d8w_8 as shipped (one accumulation sweep)

Cases: the reference's own data/dem.tif (104 x 124, 90 m, nodata -9999) and
seeded synthetic DEMs from pargo_gb300.synth, including an integer-quantised
one full of flats and ties.
"""
import argparse
import os
import struct
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def read_tiff_f32(path):
    """Minimal reader for an uncompressed, strip-organised float32 GeoTIFF.
    Returns (array, nodata, cellsize)."""
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
    cols, rows = tags[256][0], tags[257][0]
    assert tags[258][0] == 32 and tags[259][0] == 1 and tags.get(339, (3,))[0] == 3, "float32 uncompressed only"
    data = b"".join(b[o:o + c] for o, c in zip(tags[273], tags[279]))
    arr = np.frombuffer(data, dtype=bo + "f4", count=rows * cols).reshape(rows, cols).astype(np.float32)
    nodata = float(tags[42113]) if 42113 in tags else -9999.0
    cellsize = tags[33550][0] if 33550 in tags else 1.0
    return arr, nodata, cellsize


def cases(reference_root):
    from pargo_gb300 import synth
    out = []
    dem, nd, cs = read_tiff_f32(os.path.join(reference_root, "data", "dem.tif"))
    out.append(("demtif", dem, nd, cs))
    out.append(("fbm_slope", synth.slope_dem(61, 83, seed=0), -9999.0, 30.0))
    out.append(("fbm_hydro", synth.hydro_dem(96, 130, seed=11), -9999.0, 30.0))
    q = np.round(synth.fbm(40, 52, 5, 0.7, 0.0, 12.0)).astype(np.float32)  # integer metres: flats and ties
    q[17:22, 20:30] = 3.0
    q[0, :] = -9999.0
    out.append(("quantised", q, -9999.0, 10.0))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-root", default=os.environ.get("PARGO_REFERENCE_ROOT", "/root/reference"))
    args = ap.parse_args()
    os.environ["PARGO_REFERENCE_ROOT"] = args.reference_root
    import oracle
    from oracle import build as obuild
    obuild.REFERENCE_ROOT = args.reference_root
    obuild.build()
    R = oracle.Reference()
    for name, dem, nd, cs in cases(args.reference_root):
        rec = {"dem": dem, "nodata": np.float64(nd), "cellsize": np.float64(cs)}
        for m in range(7):
            rec["slope_m%d" % m] = R.slope(dem, nd, cs, method=m)
        rec["d8_8"] = R.d8(dem, nd, cs, dir_type=8)
        rec["d8_256"] = R.d8(dem, nd, cs, dir_type=256)
        w, sweeps = R.fill(dem, nd, cs)
        rec["fill"] = w
        rec["fill_sweeps"] = np.int64(sweeps)
        d8w = R.d8(w, nd, cs, dir_type=8)
        rec["d8w_8"] = d8w
        rec["sca_conv"], _ = R.sca(d8w, nd, cs, converged=True)
        rec["sca_ship"], _ = R.sca(d8w, nd, cs, converged=False)
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **rec)
        print("wrote", path, dem.shape, "fill sweeps", sweeps)


if __name__ == "__main__":
    main()
