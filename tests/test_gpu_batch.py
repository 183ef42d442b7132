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
