"""MFD-md on the GPU: flow partition weights (pargo_mfd, FP32) and the MFD
specific catchment area (pargo_sca_mfd, FP64 sums) against the oracle, which
is pinned bit for bit to the reference MFDOperator and scamfdmd SCAOperator
(tests/test_oracle.py).

Tolerances: weights |gpu - ref| <= 1e-5 |ref| + 1e-6 (FP32 powf against FP64
pow; the set of flow neighbours, i.e. which weights are zero, must match
exactly); SCA given the oracle's weights: bit-identical; SCA of the whole
chain (GPU weights in): |gpu - ref| <= 1e-4 |ref|."""
import numpy as np
import pytest

from conftest import bits_equal
from gpu_helpers import dev, empty_dev, host
from pargo_gb300 import abi, synth

pytestmark = pytest.mark.gpu
ND = -9999.0


def _dem(oracle_lib, shape, seed, filled=True):
    d = synth.hydro_dem(shape[0], shape[1], seed=seed, blob_fraction=0.05)
    if filled:
        d = oracle_lib.fill(d, ND).astype(np.float32)
    d[shape[0] // 2:shape[0] // 2 + 3, 10:20] = d[shape[0] // 2, 10]   # an exact flat
    return d


def _weights_gpu(ctx, dem, cs, e, dtype=np.float64, host_io=False):
    if host_io:
        ws = [np.empty(dem.shape, dtype) for _ in range(8)]
        ctx.mfd(abi.raster(dem, ND, cs), [abi.raster(w, ND) for w in ws], slp_exp=e)
        return np.stack(ws).astype(np.float64)
    ws = [empty_dev(dem.shape, dtype) for _ in range(8)]
    ctx.mfd(abi.raster(dev(dem), ND, cs), [abi.raster(w, ND) for w in ws], slp_exp=e)
    return np.stack([host(w) for w in ws]).astype(np.float64)


def _weights_close(g, r):
    nd = r == ND
    assert np.array_equal(g == ND, nd)
    assert np.array_equal(g == 0.0, r == 0.0)
    ok = ~nd
    err = np.abs(g[ok] - r[ok])
    assert (err <= 1e-5 * np.abs(r[ok]) + 1e-6).all(), err.max()


@pytest.mark.parametrize("e", [-1.0, 0.0, 0.5, 1.1])
def test_weights_against_oracle(e, ctx, oracle_lib):
    dem = _dem(oracle_lib, (203, 317), 71)
    _weights_close(_weights_gpu(ctx, dem, 30.0, e), oracle_lib.mfd(dem, ND, 30.0, e))


@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_weights_float64_dem_and_host_buffers(dt, ctx, oracle_lib):
    d = synth.hydro_dem(150, 190, seed=72)
    w = oracle_lib.fill(d, ND)             # float64 levels, drops of order the gap
    ref = oracle_lib.mfd(w, ND, 10.0, 1.1)
    _weights_close(_weights_gpu(ctx, w, 10.0, 1.1, dtype=dt, host_io=True), ref)


def test_sca_bit_exact_given_oracle_weights(ctx, oracle_lib):
    for shape, seed, filled in [((203, 317), 73, True), ((120, 260), 74, False), ((3, 3), 75, True)]:
        dem = _dem(oracle_lib, shape, seed, filled) if min(shape) > 8 else np.full(shape, 5.0, np.float32)
        w = oracle_lib.mfd(dem, ND, 30.0, 1.1)
        ref = oracle_lib.sca_mfd(w, ND)
        out = empty_dev(shape, np.float64)
        ctx.sca_mfd([abi.raster(dev(w[q]), ND) for q in range(8)], abi.raster(out, ND))
        g = host(out)
        assert np.array_equal(g.view(np.int64), ref.view(np.int64)), (shape, np.abs(g - ref).max())


@pytest.mark.parametrize("shape", [(1100, 70), (45, 1500), (33, 34), (34, 33)])
@pytest.mark.parametrize("dt", [np.float32, np.float64])
def test_sca_bands_tall_wide_and_edge_sizes(shape, dt, ctx, oracle_lib):
    """Many 32-row bands over short rows, one band over long rows, and sizes
    around one band (33 and 34 rows: a second band of one work row or none),
    with float32 and float64 weights: bit for bit against the oracle."""
    dem = _dem(oracle_lib, shape, 77 + shape[0] % 13)
    w = oracle_lib.mfd(dem, ND, 30.0, 1.1).astype(dt)
    ref = oracle_lib.sca_mfd(w.astype(np.float64), ND)
    out = empty_dev(shape, np.float64)
    ctx.sca_mfd([abi.raster(dev(np.ascontiguousarray(w[q])), ND) for q in range(8)], abi.raster(out, ND))
    g = host(out)
    assert np.array_equal(g.view(np.int64), ref.view(np.int64)), (shape, np.abs(g - ref).max())


def test_sca_host_buffers_float32_weights(ctx, oracle_lib):
    dem = _dem(oracle_lib, (140, 170), 76)
    w = oracle_lib.mfd(dem, ND, 30.0, 1.1).astype(np.float32)
    ref = oracle_lib.sca_mfd(w.astype(np.float64), ND)
    out = np.empty(dem.shape, np.float64)
    ctx.sca_mfd([abi.raster(np.ascontiguousarray(w[q]), ND) for q in range(8)], abi.raster(out, ND))
    assert np.array_equal(out.view(np.int64), ref.view(np.int64))


def test_chain_weights_then_sca(ctx, oracle_lib):
    dem = _dem(oracle_lib, (256, 300), 77)
    ref = oracle_lib.sca_mfd(oracle_lib.mfd(dem, ND, 30.0, 1.1), ND)
    ws = [empty_dev(dem.shape, np.float64) for _ in range(8)]
    ctx.mfd(abi.raster(dev(dem), ND, 30.0), [abi.raster(w, ND) for w in ws], slp_exp=1.1)
    out = empty_dev(dem.shape, np.float64)
    ctx.sca_mfd([abi.raster(w, ND) for w in ws], abi.raster(out, ND))
    g = host(out)
    assert np.array_equal(g == ND, ref == ND)
    ok = ref != ND
    rel = np.abs(g[ok] - ref[ok]) / np.abs(ref[ok])
    print("MFD SCA chain: max rel err %.3g" % rel.max())
    assert rel.max() <= 1e-4


def test_sca_evaluates_a_cycle_as_the_sweep_and_rejects_weights_into_nodata(ctx, oracle_lib):
    """A weight cycle is no error in the reference: its single sweep pulls
    neither cell of the cycle into the other (each still waits on the other
    when it is visited), so both keep 1.  The GPU gives the same; weights into
    a nodata cell are refused."""
    R, C = 6, 7
    w = np.zeros((8, R, C))
    w[:, 0, :] = w[:, -1, :] = w[:, :, 0] = w[:, :, -1] = ND
    # (2,2) -> east (2,3) (layer 4 = position 5) and (2,3) -> west (2,2) (layer 3 = position 3)
    w[4, 2, 2] = 1.0
    w[3, 2, 3] = 1.0
    out = empty_dev((R, C), np.float64)
    ctx.sca_mfd([abi.raster(dev(np.ascontiguousarray(w[q])), ND) for q in range(8)], abi.raster(out, ND))
    want = oracle_lib.sca_mfd(w, ND)
    assert want[2, 2] == 1.0 and want[2, 3] == 1.0
    assert bits_equal(host(out), want)
    w2 = np.zeros((8, R, C))
    w2[:, 0, :] = w2[:, -1, :] = w2[:, :, 0] = w2[:, :, -1] = ND
    w2[:, 3, 3] = ND            # a nodata cell ...
    w2[4, 3, 2] = 0.5           # ... that receives flow
    with pytest.raises(abi.PargoError):
        ctx.sca_mfd([abi.raster(dev(np.ascontiguousarray(w2[q])), ND) for q in range(8)], abi.raster(out, ND))
