"""Seeded synthetic DEM workloads (bindings to ``csrc/synth.c``).

The generators are deterministic functions of their arguments and produce
the same float32 bytes on x86-64 and aarch64 (see ``csrc/synth.c``).  The
workload helpers build the raster shapes that the focal operators are
benchmarked and tested on:

* ``slope_dem``       -- fBm DEM with a one-cell nodata border (Horn slope);
* ``hydro_dem``       -- fBm DEM with lowered pit cells and a random-walk
                         nodata blob (D8 + pit removal);
* ``batch_shapes``    -- per-raster (rows, cols, hurst) of a batch of uneven rasters;
* ``perturbed``       -- DEM plus a seeded N(0, sigma^2)-like perturbation.
"""
import ctypes
import math

import numpy as np

from . import _paths

NODATA = -9999.0

_lib = None


def _load():
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(_paths.require(_paths.SYNTH_SO))
        u64, d, i, fp = ctypes.c_uint64, ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_float)
        lib.pargo_synth_u01.argtypes = [u64, u64, u64, u64]
        lib.pargo_synth_u01.restype = d
        lib.pargo_synth_fbm.argtypes = [u64, d, d, d, i, i, fp]
        lib.pargo_synth_border.argtypes = [fp, i, i, i, ctypes.c_float]
        lib.pargo_synth_pits.argtypes = [fp, i, i, u64, d, d, ctypes.c_float]
        lib.pargo_synth_blob.argtypes = [fp, i, i, u64, d, ctypes.c_float]
        lib.pargo_synth_blob.restype = ctypes.c_int64
        lib.pargo_synth_perturb.argtypes = [fp, fp, i, i, u64, d, ctypes.c_float]
        _lib = lib
    return _lib


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def fbm(rows, cols, seed, hurst, lo, hi):
    """Diamond-square fBm surface, rescaled to [lo, hi], float32 (rows, cols)."""
    out = np.empty((rows, cols), np.float32)
    rc = _load().pargo_synth_fbm(seed, hurst, lo, hi, rows, cols, _fp(out))
    if rc:
        raise RuntimeError("pargo_synth_fbm rc=%d" % rc)
    return out


def u01(seed, stream, i, j):
    return _load().pargo_synth_u01(seed, stream, i, j)


def slope_dem(rows=1024, cols=1024, seed=0, hurst=0.8, relief=2000.0, border=1):
    """fBm DEM over [0, relief] m with a `border`-cell nodata frame."""
    dem = fbm(rows, cols, seed, hurst, 0.0, relief)
    if border:
        _load().pargo_synth_border(_fp(dem), rows, cols, border, NODATA)
    return dem


def hydro_dem(rows=8192, cols=8192, seed=1, hurst=0.75, relief=3000.0, pit_fraction=0.01, pit_depth=5.0,
              blob_fraction=0.10):
    """fBm DEM with `pit_fraction` of cells lowered by U(0, pit_depth) m and a
    random-walk nodata blob covering `blob_fraction` of the raster."""
    dem = fbm(rows, cols, seed, hurst, 0.0, relief)
    lib = _load()
    if pit_fraction > 0:
        lib.pargo_synth_pits(_fp(dem), rows, cols, seed, pit_fraction, pit_depth, NODATA)
    if blob_fraction > 0:
        lib.pargo_synth_blob(_fp(dem), rows, cols, seed, blob_fraction, NODATA)
    return dem


def perturbed(dem, seed, sigma=0.5):
    out = np.empty_like(dem)
    d = np.ascontiguousarray(dem, np.float32)
    _load().pargo_synth_perturb(_fp(d), _fp(out), d.shape[0], d.shape[1], seed, sigma, NODATA)
    return out


def batch_shapes(n=512, first_seed=100, lo=256, hi=4096, hurst_lo=0.6, hurst_hi=0.9):
    """(seed, rows, cols, hurst) for a batch of independent rasters: each side
    log-uniform in [lo, hi] (drawn separately, so rasters are non-square) and
    Hurst uniform in [hurst_lo, hurst_hi]."""
    out = []
    for k in range(n):
        s = first_seed + k
        r = int(round(math.exp(math.log(lo) + (math.log(hi) - math.log(lo)) * u01(s, 0xBA7C, 0, 0))))
        c = int(round(math.exp(math.log(lo) + (math.log(hi) - math.log(lo)) * u01(s, 0xBA7C, 0, 1))))
        h = hurst_lo + (hurst_hi - hurst_lo) * u01(s, 0xBA7C, 0, 2)
        out.append((s, r, c, h))
    return out


def batch_dems(n=512, first_seed=100, relief=2000.0):
    return [slope_dem(r, c, seed=s, hurst=h, relief=relief) for (s, r, c, h) in batch_shapes(n, first_seed)]
