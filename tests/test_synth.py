"""The synthetic workload generator is deterministic, and the per-workload
edits do what their names say."""
import numpy as np

from pargo_gb300 import synth


def test_fbm_is_deterministic_and_in_range():
    a = synth.fbm(129, 100, 7, 0.8, 0.0, 2000.0)
    b = synth.fbm(129, 100, 7, 0.8, 0.0, 2000.0)
    assert np.array_equal(a, b)
    assert a.min() == 0.0 and a.max() == 2000.0
    c = synth.fbm(129, 100, 8, 0.8, 0.0, 2000.0)
    assert not np.array_equal(a, c)


def test_slope_dem_border():
    d = synth.slope_dem(50, 40, seed=0)
    assert (d[0] == synth.NODATA).all() and (d[:, -1] == synth.NODATA).all()
    assert (d[1:-1, 1:-1] != synth.NODATA).all()


def test_hydro_dem_blob_and_pits():
    base = synth.fbm(200, 180, 1, 0.75, 0.0, 3000.0)
    d = synth.hydro_dem(200, 180, seed=1)
    frac = (d == synth.NODATA).mean()
    assert 0.10 <= frac < 0.12
    valid = d != synth.NODATA
    lowered = (d < base) & valid
    assert 0.005 < lowered.sum() / valid.sum() < 0.015
    assert ((base - d)[lowered] <= 5.0 + 1e-3).all()


def test_batch_shapes():
    shapes = synth.batch_shapes(512)
    assert len(shapes) == 512
    rows = np.array([s[1] for s in shapes])
    cols = np.array([s[2] for s in shapes])
    assert rows.min() >= 256 and rows.max() <= 4096 and cols.min() >= 256 and cols.max() <= 4096
    assert (rows != cols).mean() > 0.9
    assert all(0.6 <= s[3] <= 0.9 for s in shapes)
    assert shapes == synth.batch_shapes(512)
