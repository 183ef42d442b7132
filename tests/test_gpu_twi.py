"""Topographic wetness index on the GPU (pargo_twi) against the oracle, which
is pinned to the reference TWIOperator (tests/test_oracle.py).  The GPU
computes in FP32: tolerance |gpu - ref| <= 1e-6 |ref| + 1e-6; the nodata mask
must match exactly."""
import numpy as np
import pytest

from gpu_helpers import dev, empty_dev, host
from pargo_gb300 import abi, synth

pytestmark = pytest.mark.gpu
ND = -9999.0


def _inputs(oracle_lib, shape, seed):
    dem = synth.hydro_dem(shape[0], shape[1], seed=seed)
    w = oracle_lib.fill(dem, ND)
    sl = oracle_lib.slope(w, ND, 30.0)
    sca = oracle_lib.sca(oracle_lib.d8(w, ND), ND, shipped=True)
    sl[10, 10:20] = 0.0        # flats: slope raised to 1e-7
    sl[12, 12] = 5e-8
    return sl, sca


def _close(g, r):
    g = g.astype(np.float64)
    nd = r == ND
    assert np.array_equal(g == ND, nd)
    ok = ~nd
    assert (np.abs(g[ok] - r[ok]) <= 1e-6 * np.abs(r[ok]) + 1e-6).all(), np.abs(g[ok] - r[ok]).max()


@pytest.mark.parametrize("sdt,adt,odt", [(np.float64, np.float64, np.float64), (np.float32, np.float64, np.float32),
                                         (np.float32, np.float32, np.float32)])
def test_twi_against_oracle(sdt, adt, odt, ctx, oracle_lib):
    sl, sca = _inputs(oracle_lib, (300, 411), 61)
    sl_in, sca_in = sl.astype(sdt), sca.astype(adt)
    ref = oracle_lib.twi(sl_in.astype(np.float64), sca_in.astype(np.float64), ND)
    out = empty_dev(sl.shape, odt)
    ctx.twi(abi.raster(dev(sl_in), ND), abi.raster(dev(sca_in), ND), abi.raster(out, ND))
    _close(host(out), ref)


def test_twi_host_buffers_and_odd_nodata(ctx, oracle_lib):
    sl, sca = _inputs(oracle_lib, (129, 260), 62)
    out = np.empty(sl.shape, np.float64)          # host in, host out
    ctx.twi(abi.raster(sl, ND), abi.raster(sca, ND), abi.raster(out, ND))
    _close(out, oracle_lib.twi(sl, sca, ND))
    # a nodata value that is not a float: float inputs never equal it, double inputs do
    odd = -9999.1
    sl2 = np.where(sl == ND, odd, sl)
    sca2 = np.where(sca == ND, odd, sca)
    ref = oracle_lib.twi(sl2, sca2, odd, out_nodata=odd)
    out2 = empty_dev(sl.shape, np.float64)
    ctx.twi(abi.raster(dev(sl2), odd), abi.raster(dev(sca2), odd), abi.raster(out2, odd))
    g = host(out2)
    assert np.array_equal(g == odd, ref == odd)
    ok = ref != odd
    assert (np.abs(g[ok] - ref[ok]) <= 1e-6 * np.abs(ref[ok]) + 1e-6).all()
    f32 = sl2.astype(np.float32)
    ref32 = oracle_lib.twi(f32.astype(np.float64), sca2, odd, out_nodata=odd)
    out3 = empty_dev(sl.shape, np.float64)
    ctx.twi(abi.raster(dev(f32), odd), abi.raster(dev(sca2), odd), abi.raster(out3, odd))
    g3 = host(out3)
    assert np.array_equal(g3 == odd, ref32 == odd)
