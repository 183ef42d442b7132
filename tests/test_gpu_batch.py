"""Batched slope + D8 (one persistent launch over many uneven rasters) gives
exactly what per-raster launches give, and matches the oracle."""
import numpy as np
import pytest
import torch

from conftest import bits_equal
from gpu_helpers import d8_as_f64, dev, empty_dev, host, slope_close
from pargo_gb300 import abi, synth

pytestmark = pytest.mark.gpu


def _batch(n, first_seed, scale):
    shapes = synth.batch_shapes(n, first_seed=first_seed, lo=int(256 * scale), hi=int(4096 * scale))
    return [(s, max(r, 3), max(c, 3), h) for (s, r, c, h) in shapes]


@pytest.mark.parametrize("align", [16, 0])
def test_batch_equals_per_raster_and_oracle(align, ctx, oracle_lib):
    shapes = _batch(24, 100, 0.125)
    dems = [synth.slope_dem(r, c, seed=s, hurst=h) for (s, r, c, h) in shapes]
    dd = [dev(d, align) for d in dems]
    bs = [empty_dev(d.shape, np.float32, align) for d in dems]
    bc = [empty_dev(d.shape, np.int8, align) for d in dems]
    ctx.batch_slope_d8([abi.raster(d, -9999.0, 30.0) for d in dd], [abi.raster(s, -9999.0) for s in bs],
                       [abi.raster(c, -128) for c in bc])
    for k, dem in enumerate(dems):
        s = empty_dev(dem.shape, np.float32, align)
        c = empty_dev(dem.shape, np.int8, align)
        ctx.slope_d8(abi.raster(dd[k], -9999.0, 30.0), abi.raster(s, -9999.0), abi.raster(c, -128))
        assert bits_equal(host(bs[k]), host(s)), k
        assert bits_equal(host(bc[k]), host(c)), k
        ok, mx, _ = slope_close(host(bs[k]), oracle_lib.slope(dem, -9999.0, 30.0))
        assert ok, mx
        assert bits_equal(d8_as_f64(host(bc[k]), -128), oracle_lib.d8(dem, -9999.0))


def test_batch_mixed_outputs_and_cache(ctx, oracle_lib):
    shapes = _batch(9, 300, 0.1)
    dems = [synth.hydro_dem(r, c, seed=s) for (s, r, c, h) in shapes]
    dd = [dev(d, 16) for d in dems]
    outs = [empty_dev(d.shape, np.float64, 16) for d in dems]
    for _ in range(2):  # second call reuses the cached device tables
        ctx.batch_slope_d8([abi.raster(d, -9999.0) for d in dd], None, [abi.raster(o, -9999.0) for o in outs],
                           dir_type=256)
        for k, dem in enumerate(dems):
            assert bits_equal(host(outs[k]), oracle_lib.d8(dem, -9999.0, dir_type=256))


@pytest.mark.parametrize("outputs", ["both", "slope", "d8"])
def test_batch_strip_walk_with_nodata_and_edge_sizes(outputs, ctx, oracle_lib):
    """The batched strip walk (aligned float32 / int8 outputs, Horn, dirType 8)
    on DEMs with nodata blobs and shapes at the 48-row segment and 128-column
    strip boundaries: identical to the per-raster launches and the oracle."""
    shapes = [(3, 3), (47, 129), (48, 128), (49, 127), (97, 385), (200, 130), (143, 257), (1024, 700)]
    dems = [synth.hydro_dem(r, c, seed=11 + k) for k, (r, c) in enumerate(shapes)]
    dd = [dev(d, 16) for d in dems]
    want_s, want_c = outputs in ("both", "slope"), outputs in ("both", "d8")
    bs = [empty_dev(d.shape, np.float32, 16) for d in dems] if want_s else None
    bc = [empty_dev(d.shape, np.int8, 16) for d in dems] if want_c else None
    ctx.batch_slope_d8([abi.raster(d, -9999.0, 30.0) for d in dd], [abi.raster(s, -9999.0) for s in bs] if bs else None,
                       [abi.raster(c, -128) for c in bc] if bc else None)
    for k, dem in enumerate(dems):
        if want_s:
            ok, mx, _ = slope_close(host(bs[k]), oracle_lib.slope(dem, -9999.0, 30.0))
            assert ok, (k, mx)
        if want_c:
            assert bits_equal(d8_as_f64(host(bc[k]), -128), oracle_lib.d8(dem, -9999.0)), k


def _np_queue(dems, nodata_load, valid_load, seg_rows=48, seg_cols=128):
    """The queue by intensity, restated: segment loads counted with
    |v - nodata| > 1e-7 as valid, summed per raster, rasters heaviest first
    (a stable sort of the rasters by size, largest first), each raster's
    segments in order."""
    korder = sorted(range(len(dems)), key=lambda i: -dems[i].size)   # Python's sort is stable
    per = []
    for k in korder:
        d = dems[k].astype(np.float64)
        valid = np.abs(d - (-9999.0)) > 1e-7
        R, C = d.shape
        ns = (C + seg_cols - 1) // seg_cols
        nb = (R + seg_rows - 1) // seg_rows
        items = []
        for l in range(ns * nb):
            x0, y0 = (l % ns) * seg_cols, (l // ns) * seg_rows
            v = valid[y0:y0 + seg_rows, x0:x0 + seg_cols]
            items.append((k, l, float(v.sum()) * valid_load + float(v.size - v.sum()) * nodata_load))
        per.append(items)
    order = sorted(range(len(per)), key=lambda j: -sum(it[2] for it in per[j]))
    return [it for j in order for it in per[j]]


@pytest.mark.parametrize("loads", [(0.0, 1.0), (3.0, 1.0)])
def test_batch_queue_by_intensity_matches_restatement(loads, ctx):
    """The device-counted segment loads and the queue order equal a numpy
    restatement of the intensity-ratio estimate on DEMs with nodata blobs."""
    shapes = [(300, 700), (97, 130), (1024, 129), (48, 128), (49, 257), (500, 500)]
    dems = [synth.hydro_dem(r, c, seed=400 + k, blob_fraction=0.15) for k, (r, c) in enumerate(shapes)]
    dd = [dev(d, 16) for d in dems]
    ras, seg, ld = ctx.batch_queue([abi.raster(d, -9999.0) for d in dd], nodata_load=loads[0], valid_load=loads[1])
    want = _np_queue(dems, *loads)
    assert len(ras) == len(want)
    assert np.array_equal(ld, np.array([w[2] for w in want]))
    assert np.array_equal(ras, np.array([w[0] for w in want]))
    assert np.array_equal(seg, np.array([w[1] for w in want]))
    rl = [ld[ras == k].sum() for k in list(dict.fromkeys(ras.tolist()))]
    assert (np.diff(rl) <= 0).all()                            # rasters heaviest first
    r2, s2, l2 = ctx.batch_queue([abi.raster(d, -9999.0) for d in dd], order=abi.BATCH_BY_SIZE)
    korder = sorted(range(len(dems)), key=lambda i: -dems[i].size)
    assert list(dict.fromkeys(r2.tolist())) == korder       # raster by raster, largest first


@pytest.mark.parametrize("order,loads", [(0, (0.0, 1.0)), (0, (5.0, 1.0)), (1, (0.0, 1.0))])
def test_batch_outputs_do_not_depend_on_the_queue_order(order, loads, ctx, oracle_lib):
    shapes = _batch(14, 500, 0.1)
    dems = [synth.hydro_dem(r, c, seed=s, blob_fraction=0.12) for (s, r, c, h) in shapes]
    dd = [dev(d, 16) for d in dems]
    bs = [empty_dev(d.shape, np.float32, 16) for d in dems]
    bc = [empty_dev(d.shape, np.int8, 16) for d in dems]
    ctx.batch_slope_d8([abi.raster(d, -9999.0, 30.0) for d in dd], [abi.raster(s, -9999.0) for s in bs],
                       [abi.raster(c, -128) for c in bc], order=order, nodata_load=loads[0], valid_load=loads[1])
    for k, dem in enumerate(dems):
        ok, mx, _ = slope_close(host(bs[k]), oracle_lib.slope(dem, -9999.0, 30.0))
        assert ok, (k, mx)
        assert bits_equal(d8_as_f64(host(bc[k]), -128), oracle_lib.d8(dem, -9999.0)), k
