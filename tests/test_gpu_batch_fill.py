"""Batched pit removal (pargo_batch_fill): many uneven rasters in one
persistent relaxation give, raster by raster, exactly the oracle's levels and
exactly what pargo_fill gives -- float32 and float64 DEMs, float64 and float32
outputs, padded pitches, rasters down to 3 x 3, nodata blobs, and batches
whose nodata values differ (filled one by one)."""
import numpy as np
import pytest

from conftest import bits_equal
from gpu_helpers import dev, empty_dev, host
from pargo_gb300 import abi, synth

pytestmark = pytest.mark.gpu

ND = -9999.0


def _shapes():
    shapes = synth.batch_shapes(40, first_seed=700, lo=3, hi=700)
    return [(3, 3), (3, 257), (211, 3), (64, 64), (33, 95)] + [(r, c) for (_, r, c, _) in shapes]


@pytest.mark.parametrize("gap,out_dtype,align", [(1e-3, np.float64, 16), (5e-4, np.float32, 0)])
def test_batch_fill_matches_oracle_and_single_fills(gap, out_dtype, align, ctx, oracle_lib):
    dems = [synth.hydro_dem(r, c, seed=900 + k, blob_fraction=0.08) for k, (r, c) in enumerate(_shapes())]
    dd = [dev(d, align) for d in dems]
    ww = [empty_dev(d.shape, out_dtype, align) for d in dems]
    st = ctx.batch_fill([abi.raster(d, ND, 30.0) for d in dd], [abi.raster(w, ND) for w in ww], gap=gap)
    raised = 0
    for k, dem in enumerate(dems):
        ref = oracle_lib.fill(dem, ND, gap=gap)
        got = host(ww[k])
        if out_dtype == np.float64:
            assert bits_equal(got, ref), k
        else:
            assert np.array_equal(got, ref.astype(np.float32)), k
        one = empty_dev(dem.shape, out_dtype, align)
        ctx.fill(abi.raster(dd[k], ND, 30.0), abi.raster(one, ND), gap=gap)
        assert np.array_equal(host(one).view(np.uint8), got.view(np.uint8)), k
        raised += int((ref[ref != ND] > dem[ref != ND]).sum())
    assert st.rounds == 1 and st.tile_visits > 0
    assert st.raised_cells == raised


def test_batch_fill_float64_dems_and_second_call(ctx, oracle_lib):
    dems = [synth.hydro_dem(r, c, seed=950 + k).astype(np.float64) for k, (r, c) in
            enumerate([(120, 340), (257, 64), (5, 5), (300, 301)])]
    dd = [dev(d, 16) for d in dems]
    for _ in range(2):   # the second call reuses the context's mosaic and tables
        ww = [empty_dev(d.shape, np.float64, 16) for d in dems]
        ctx.batch_fill([abi.raster(d, ND) for d in dd], [abi.raster(w, ND) for w in ww], gap=1e-3)
        for k, dem in enumerate(dems):
            assert bits_equal(host(ww[k]), oracle_lib.fill(dem.astype(np.float32), ND, gap=1e-3)), k


def test_batch_fill_with_differing_nodata_fills_one_by_one(ctx, oracle_lib):
    dems = [synth.hydro_dem(90, 130, seed=960), synth.hydro_dem(64, 70, seed=961)]
    dems[1] = np.where(dems[1] == ND, np.float32(-32768.0), dems[1]).astype(np.float32)
    nds = [ND, -32768.0]
    dd = [dev(d) for d in dems]
    ww = [empty_dev(d.shape, np.float64) for d in dems]
    ctx.batch_fill([abi.raster(d, nd) for d, nd in zip(dd, nds)], [abi.raster(w, nd) for w, nd in zip(ww, nds)])
    for k, dem in enumerate(dems):
        assert bits_equal(host(ww[k]), oracle_lib.fill(dem, nds[k])), k


def test_batch_fill_rejects_host_rasters(ctx):
    dem = synth.hydro_dem(20, 20, seed=1)
    out = np.empty(dem.shape, np.float64)
    with pytest.raises(abi.PargoError) as e:
        ctx.batch_fill([abi.raster(dem, ND)], [abi.raster(out, ND)])
    assert e.value.status_name == "PARGO_ERR_INVALID_ARG"
