"""Size-independent exactness check of a pit-removal result (test helper).

The reference's relaxation (apps/hydrology/pitremove/pitRemoveOperator.cpp:
26-72, swept by gpro/rasterOperator.h:169-219) stops at the greatest level
surface W <= init_level that no visit lowers.  On every valid work cell c
with dem(c) < init_level that surface satisfies

    W(c) = dem(c)                                          if a neighbour's level is nodata,
    W(c) = min(init_level, max(dem(c), min_n W(n) + gap))  otherwise,

with W(n) + gap the IEEE double sum.  Any W with dem <= W < init_level that
satisfies these equations everywhere IS the reference's surface: W is then a
surface no visit lowers, so W <= the reference's; and among the cells where
the two differ take one whose W is least -- the neighbour that sets it is
strictly lower (fl(x + gap) > x for every level here), so the surfaces agree
on that neighbour, and the reference's own update then puts the cell at or
below W.  Checking the equations cell by cell (numpy's float64 add is the
IEEE sum) therefore proves bit equality with the reference in O(N) time, one
band of rows at a time, at sizes where the oracle itself would take minutes.
"""
import numpy as np

EPS_HYDRO = 1e-6  # pitRemoveOperator.cpp:40,53,59 (Eps of pitRemoveOperator.h)


def fill_fixpoint_mismatches(dem, W, nodata=-9999.0, gap=5e-4, init_level=10000.0, band=2048):
    """Number of cells where W breaks the equations above, plus ring cells not
    at nodata and valid cells at or above init_level (0 = W is the reference's
    result).  dem: float32 or float64 (rows, cols); W: float64 (rows, cols)."""
    dem = np.asarray(dem)
    W = np.asarray(W, np.float64)
    R, C = dem.shape
    assert W.shape == (R, C) and R >= 3 and C >= 3
    ring = np.concatenate([W[0], W[-1], W[1:-1, 0], W[1:-1, -1]])
    bad = int((ring != nodata).sum())
    for r0 in range(1, R - 1, band):
        r1 = min(r0 + band, R - 1)                 # work rows r0 .. r1-1
        h = r1 - r0
        z = dem[r0:r1, 1:-1].astype(np.float64)
        w = W[r0:r1, 1:-1]
        win = W[r0 - 1:r1 + 1]                     # levels of the band with a one-cell halo (ring included)
        valid = np.abs(z - nodata) > EPS_HYDRO
        m = np.full(z.shape, np.inf)
        nd_nbr = np.zeros(z.shape, bool)
        for a in (0, 1, 2):
            for b in (0, 1, 2):
                if a == 1 and b == 1:
                    continue
                wn = win[a:a + h, b:b + C - 2]
                isnd = np.abs(wn - nodata) < EPS_HYDRO
                nd_nbr |= isnd
                m = np.minimum(m, np.where(isnd, np.inf, wn))
        expect = np.where(nd_nbr, z, np.minimum(init_level, np.maximum(z, m + gap)))
        expect = np.where(z >= init_level, init_level, expect)
        expect = np.where(valid, expect, nodata)
        bad += int((w.view(np.int64) != expect.view(np.int64)).sum())
        bad += int((valid & (w >= init_level) & (z < init_level)).sum())
    return bad
