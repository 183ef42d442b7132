"""Pit removal and SCA on the GPU through the C ABI, bit-exact against the
reference (golden fixtures) and the pinned oracle (larger inputs), plus the
size-independent properties checked at the full workload sizes."""
import numpy as np
import pytest
import torch

from conftest import GOLDEN_CASES, bits_equal, load_golden, near_zero_dem
from gpu_helpers import d8_as_f64, dev, empty_dev, host, ref_noise_floor, slope_close
from pargo_gb300 import abi, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_golden_fill_bit_exact(case, ctx):
    g = load_golden(case)
    dem, nd = g["dem"], float(g["nodata"])
    w = empty_dev(dem.shape, np.float64)
    stats = ctx.fill(abi.raster(dev(dem), nd), abi.raster(w, nd))
    assert bits_equal(host(w), g["fill"])
    assert stats.raised_cells == int((g["fill"] > dem.astype(np.float64)).sum())
    w32 = np.empty(dem.shape, np.float32)   # host output, float32: the reference values rounded
    ctx.fill(abi.raster(dem, nd), abi.raster(w32, nd))
    assert np.array_equal(w32, g["fill"].astype(np.float32))


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_golden_sca_both_contracts(case, ctx):
    g = load_golden(case)
    d8, nd = g["d8w_8"], float(g["nodata"])
    for contract, key in ((abi.SCA_CONVERGED, "sca_conv"), (abi.SCA_SHIPPED, "sca_ship")):
        out = empty_dev(d8.shape, np.float64)
        ctx.sca(abi.raster(dev(d8), nd), abi.raster(out, nd), contract=contract)
        assert bits_equal(host(out), g[key]), key
        codes = np.where(d8 == nd, -128, d8).astype(np.int8)   # int8 codes, -128 sentinel
        out2 = np.empty(d8.shape, np.float64)
        ctx.sca(abi.raster(codes, -128), abi.raster(out2, nd), contract=contract)
        assert bits_equal(out2, g[key]), key + " (int8 input)"


@pytest.mark.parametrize("seed,shape", [(31, (300, 411)), (32, (513, 257)), (33, (1000, 1000))])
def test_pipeline_against_oracle(seed, shape, ctx, oracle_lib):
    """fill -> D8 (on the float64 levels) -> SCA, device-resident, vs the oracle."""
    dem = synth.hydro_dem(shape[0], shape[1], seed=seed)
    nd = -9999.0
    w = empty_dev(shape, np.float64)
    ctx.fill(abi.raster(dev(dem), nd), abi.raster(w, nd))
    wref = oracle_lib.fill(dem, nd)
    assert bits_equal(host(w), wref)
    c = empty_dev(shape, np.int8)
    ctx.d8(abi.raster(w, nd), abi.raster(c, -128))
    d8ref = oracle_lib.d8(wref, nd)
    assert bits_equal(d8_as_f64(host(c), -128), d8ref)
    for contract, shipped in ((abi.SCA_CONVERGED, False), (abi.SCA_SHIPPED, True)):
        out = empty_dev(shape, np.float64)
        ctx.sca(abi.raster(c, -128), abi.raster(out, nd), contract=contract)
        assert bits_equal(host(out), oracle_lib.sca(d8ref, nd, shipped=shipped))
    # slope on the float64 levels (integer-key path) against the FP64 oracle, stated
    s = empty_dev(shape, np.float32)
    ctx.slope(abi.raster(w, nd, 30.0), abi.raster(s, nd))
    ok, mx, mean = slope_close(host(s), oracle_lib.slope(wref, nd, 30.0), atol=ref_noise_floor(wref, 30.0))
    assert ok, mx
    print("slope error vs FP64 oracle, filled %dx%d levels, float64-input kernel: max rel %.3e, mean rel %.3e"
          % (shape[0], shape[1], mx, mean))


def test_fill_options_and_round_cap(ctx, oracle_lib):
    dem = synth.hydro_dem(200, 260, seed=41)
    w = empty_dev(dem.shape, np.float64)
    ctx.fill(abi.raster(dev(dem), -9999.0), abi.raster(w, -9999.0), gap=1e-3)
    assert bits_equal(host(w), oracle_lib.fill(dem, -9999.0, gap=1e-3))
    big = synth.hydro_dem(1024, 1024, seed=42, blob_fraction=0.0)
    wb = empty_dev(big.shape, np.float64)
    with pytest.raises(abi.PargoError) as e:
        ctx.fill(abi.raster(dev(big), -9999.0), abi.raster(wb, -9999.0), max_rounds=2)
    assert e.value.status_name == "PARGO_ERR_NOT_CONVERGED"
    # the context stays usable, and an uncapped run converges to the oracle's bytes
    st = ctx.fill(abi.raster(dev(big), -9999.0), abi.raster(wb, -9999.0))
    assert st.rounds == 1 and st.tile_visits > 32 * 32   # one persistent launch, tiles visited again
    assert bits_equal(host(wb), oracle_lib.fill(big, -9999.0))


def test_fill_persistent_and_round_forms_agree(ctx, oracle_lib, monkeypatch):
    """The persistent launch (device work queue) and the round launches reach
    the same bytes as the oracle; the persistent form is one launch."""
    dem = synth.hydro_dem(700, 900, seed=43)
    ref = oracle_lib.fill(dem, -9999.0, gap=1e-3)
    w = empty_dev(dem.shape, np.float64)
    st = ctx.fill(abi.raster(dev(dem), -9999.0), abi.raster(w, -9999.0), gap=1e-3)
    assert st.rounds == 1 and st.tile_visits > 0
    assert bits_equal(host(w), ref)
    monkeypatch.setenv("PARGO_FILL_ROUNDS", "1")
    w2 = empty_dev(dem.shape, np.float64)
    st2 = ctx.fill(abi.raster(dev(dem), -9999.0), abi.raster(w2, -9999.0), gap=1e-3)
    assert st2.rounds > 1
    assert bits_equal(host(w2), ref)


def test_fill_edge_cases(ctx, oracle_lib):
    for dem in (np.full((3, 3), 5.0, np.float32), np.full((50, 70), -9999.0, np.float32),
                np.full((64, 64), 7.0, np.float32)):
        w = empty_dev(dem.shape, np.float64)
        ctx.fill(abi.raster(dev(dem), -9999.0), abi.raster(w, -9999.0))
        assert bits_equal(host(w), oracle_lib.fill(dem, -9999.0))
    # a single deep pit in a cone, and a closed bowl
    y, x = np.mgrid[0:65, 0:65]
    bowl = (np.hypot(y - 32, x - 32)).astype(np.float32) * -1.0 + 100.0
    bowl[32, 32] = 0.0
    w = empty_dev(bowl.shape, np.float64)
    ctx.fill(abi.raster(dev(bowl), -9999.0), abi.raster(w, -9999.0))
    assert bits_equal(host(w), oracle_lib.fill(bowl, -9999.0))


def _maze(rows, cols, corridor=3, wall=1, floor=10.0, top=1000.0, sill=50.0):
    """A closed serpentine corridor (floor below the sill) that leaves the
    raster only through one sill cell next to the border: every corridor
    level is sill + k gaps, k its path length from the sill, so the front has
    to cross tiles back and forth along the whole path."""
    dem = np.full((rows, cols), top, np.float32)
    period = corridor + wall
    lanes = list(range(2, rows - 1 - corridor, period))  # lane k: rows r0 .. r0+corridor-1, clear of the ring
    for k, r0 in enumerate(lanes):
        dem[r0:r0 + corridor, 2:cols - 2] = floor
        if k + 1 < len(lanes):  # the bend to the next lane, on alternating sides
            c = cols - 2 - corridor if k % 2 == 0 else 2
            dem[r0 + corridor:r0 + period, c:c + corridor] = floor
    dem[2:2 + corridor, 1] = sill
    return dem


@pytest.mark.parametrize("shape", [(131, 97), (515, 517)])
def test_fill_long_serpentine_path(shape, ctx, oracle_lib):
    """Levels set by one path of thousands of cells through every tile row:
    the tile queue, the halo-change marks and the at-once re-visits must carry
    the front the whole way; the levels bit-exact against the oracle."""
    dem = _maze(*shape)
    ref = oracle_lib.fill(dem, -9999.0, gap=1e-3)
    assert (ref > dem).sum() > dem.size // 2
    w = empty_dev(dem.shape, np.float64)
    st = ctx.fill(abi.raster(dev(dem), -9999.0), abi.raster(w, -9999.0), gap=1e-3)
    assert bits_equal(host(w), ref)
    tiles = ((shape[0] + 31) // 32) * ((shape[1] + 31) // 32)
    assert st.tile_visits > tiles


@pytest.mark.parametrize("gap", [1e-3, 2.0 ** -10, 3 * 2.0 ** -12, 5e-4])
def test_fill_levels_near_zero(gap, ctx, oracle_lib):
    dem = near_zero_dem(96, 130, seed=7)
    ref = oracle_lib.fill(dem, -9999.0, gap=gap)
    gs, _ = oracle_lib.fill_gs(dem, -9999.0, gap=gap)
    assert bits_equal(ref, gs)
    assert (ref > dem).any()
    w = empty_dev(dem.shape, np.float64)
    ctx.fill(abi.raster(dev(dem), -9999.0), abi.raster(w, -9999.0), gap=gap)
    assert bits_equal(host(w), ref)
    w64 = empty_dev(dem.shape, np.float64)   # float64 DEM: the same values, the same levels
    ctx.fill(abi.raster(dev(dem.astype(np.float64)), -9999.0), abi.raster(w64, -9999.0), gap=gap)
    assert bits_equal(host(w64), ref)


def test_sca_cycle_is_reported(ctx):
    """Two cells draining into each other are excluded by the reference rule;
    a 4-cycle is not, and its in-degrees never clear."""
    d8 = np.full((8, 8), -1.0)
    d8[0, :] = d8[-1, :] = d8[:, 0] = d8[:, -1] = -9999.0
    d8[3, 3], d8[3, 4], d8[4, 4], d8[4, 3] = 5, 7, 3, 1   # E, S, W, N: a loop
    out = np.empty(d8.shape, np.float64)
    with pytest.raises(abi.PargoError) as e:
        ctx.sca(abi.raster(d8, -9999.0), abi.raster(out, -9999.0))
    assert e.value.status_name == "PARGO_ERR_CYCLE"


@pytest.mark.parametrize("shape", [(1500, 1700), (130, 4000), (4000, 70)])
def test_sca_tiles_against_oracle(shape, ctx, oracle_lib):
    """SCA across many 64 x 64 tiles (rivers crossing tile borders, partial
    edge tiles, thin rasters), both contracts, against the oracle."""
    dem = synth.hydro_dem(shape[0], shape[1], seed=17, blob_fraction=0.05)
    w = oracle_lib.fill(dem, -9999.0, gap=1e-3)
    d8 = oracle_lib.d8(w, -9999.0)
    codes = np.where(d8 == -9999.0, -128, d8).astype(np.int8)
    for contract, shipped in ((abi.SCA_CONVERGED, False), (abi.SCA_SHIPPED, True)):
        out = empty_dev(shape, np.float64)
        ctx.sca(abi.raster(dev(codes), -128), abi.raster(out, -9999.0), contract=contract)
        assert bits_equal(host(out), oracle_lib.sca(d8, -9999.0, shipped=shipped)), contract


def test_sca_cycle_across_tiles_and_ring_inflow(ctx):
    d8 = np.full((130, 130), 6.0)   # every cell drains SW ... into the ring
    d8[0, :] = d8[-1, :] = d8[:, 0] = d8[:, -1] = -9999.0
    cyc = d8.copy()
    # a 4-cycle on the corner of four tiles: (63,63) E, (63,64) S, (64,64) W, (64,63) N
    cyc[63, 63], cyc[63, 64], cyc[64, 64], cyc[64, 63] = 5, 7, 3, 1
    out = np.empty(cyc.shape, np.float64)
    with pytest.raises(abi.PargoError) as e:
        ctx.sca(abi.raster(cyc, -9999.0), abi.raster(out, -9999.0))
    assert e.value.status_name == "PARGO_ERR_CYCLE"
    ring = d8.copy()
    ring[0, 5] = 7.0   # a ring cell that names a work cell below it
    with pytest.raises(abi.PargoError) as e:
        ctx.sca(abi.raster(ring, -9999.0), abi.raster(out, -9999.0))
    assert e.value.status_name == "PARGO_ERR_CYCLE"
    ctx.sca(abi.raster(d8, -9999.0), abi.raster(out, -9999.0))   # the context stays usable
    assert out[1:-1, 1:-1].min() == 1.0


def test_full_size_fill_properties(ctx, oracle_lib):
    """8192^2 (the D8 + fill workload): the result is a fixpoint of the
    reference update, no level is below the DEM, and a 2048^2 crop run on its
    own matches the oracle bit for bit."""
    dem = synth.hydro_dem(8192, 8192, seed=1)
    nd = -9999.0
    w = empty_dev(dem.shape, np.float64)
    stats = ctx.fill(abi.raster(dev(dem), nd), abi.raster(w, nd))
    W = host(w)
    del w
    torch.cuda.empty_cache()
    valid = W != nd
    z = dem.astype(np.float64)
    assert (W[valid] >= z[valid]).all()
    assert stats.raised_cells == int((W[valid] > z[valid]).sum())
    # one more reference visit of every cell changes nothing
    lv = np.where(valid, W, np.inf)
    m = np.full(W.shape, np.inf)
    has_nd = np.zeros(W.shape, bool)
    for a in (-1, 0, 1):
        for b in (-1, 0, 1):
            if a == 0 and b == 0:
                continue
            sh = np.full(W.shape, np.inf)
            sh[max(a, 0):W.shape[0] + min(a, 0), max(b, 0):W.shape[1] + min(b, 0)] = \
                lv[max(-a, 0):W.shape[0] + min(-a, 0), max(-b, 0):W.shape[1] + min(-b, 0)]
            m = np.minimum(m, sh)
            has_nd |= np.isinf(sh)
    inner = np.zeros(W.shape, bool)
    inner[1:-1, 1:-1] = True
    act = inner & valid & (W > z)
    up = m + 0.0005
    new = np.where(has_nd | (up <= z), z, np.minimum(W, up))
    assert np.array_equal(new[act], W[act])
    crop = np.ascontiguousarray(dem[3000:5048, 1000:3048])
    wc = np.empty(crop.shape, np.float64)
    ctx.fill(abi.raster(crop, nd), abi.raster(wc, nd))
    assert bits_equal(wc, oracle_lib.fill(crop, nd))


def test_full_size_sca_conservation(ctx):
    """16384^2 SCA workload (filled fBm, 10 m): every valid cell is counted in
    exactly one terminal cell's catchment, so the terminal totals sum to the
    number of valid cells."""
    dem = synth.slope_dem(16384, 16384, seed=2, hurst=0.8, relief=2000.0)
    nd = -9999.0
    w = empty_dev(dem.shape, np.float64)
    ctx.fill(abi.raster(dev(dem), nd, 10.0), abi.raster(w, nd))
    c = empty_dev(dem.shape, np.int8)
    ctx.d8(abi.raster(w, nd, 10.0), abi.raster(c, -128))
    del w
    torch.cuda.empty_cache()
    out = empty_dev(dem.shape, np.float64)
    ctx.sca(abi.raster(c, -128), abi.raster(out, nd))
    codes = host(c).astype(np.int64)
    sca = host(out)
    valid = codes != -128
    valid[-2, -2] = valid[-2, -2]  # the last work cell is nodata in D8 output here
    rows, cols = codes.shape
    r, q = np.nonzero(valid)
    k = codes[r, q]
    flows = (k >= 0) & (k != 4)
    tr = np.where(flows, r + k // 3 - 1, -1)
    tq = np.where(flows, q + k % 3 - 1, -1)
    inside = flows & (tr >= 1) & (tq >= 1) & (tr <= rows - 2) & (tq <= cols - 2)
    tgt_valid = np.zeros_like(inside)
    tgt_valid[inside] = valid[tr[inside], tq[inside]]
    terminal = ~tgt_valid
    assert int(sca[r[terminal], q[terminal]].sum()) == int(valid.sum())


@pytest.mark.parametrize("host_io", [False, True])
def test_hydro_pipeline_matches_separate_calls_and_oracle(host_io, ctx, oracle_lib):
    """pargo_hydro_pipeline (fill -> slope + D8 on the float64 levels -> SCA)
    equals the oracle's chain, with device or host buffers."""
    dem = synth.hydro_dem(700, 530, seed=51)
    nd = -9999.0
    shape = dem.shape
    if host_io:
        src = dem
        w, s, c, a = (np.empty(shape, np.float32), np.empty(shape, np.float32), np.empty(shape, np.int8),
                      np.empty(shape, np.float64))
        get = lambda x: x
    else:
        src = dev(dem)
        w, s, c, a = (empty_dev(shape, np.float32), empty_dev(shape, np.float32), empty_dev(shape, np.int8),
                      empty_dev(shape, np.float64))
        get = host
    st = ctx.hydro_pipeline(abi.raster(src, nd, 30.0), wdem=abi.raster(w, nd), slope=abi.raster(s, nd),
                            d8=abi.raster(c, -128), sca=abi.raster(a, nd), gap=1e-3)
    wref = oracle_lib.fill(dem, nd, gap=1e-3)
    assert np.array_equal(get(w), wref.astype(np.float32))
    d8ref = oracle_lib.d8(wref, nd)
    assert bits_equal(d8_as_f64(get(c), -128), d8ref)
    from gpu_helpers import ref_noise_floor, slope_close
    ok, mx, _ = slope_close(get(s), oracle_lib.slope(wref, nd, 30.0), nd, atol=ref_noise_floor(wref, 30.0))
    assert ok, mx
    assert bits_equal(get(a), oracle_lib.sca(d8ref, nd))
    assert st.active_rounds >= 1 and st.rounds >= st.active_rounds and st.rounds_ms > 0
    assert st.raised_cells == int((wref[wref != nd] > dem[wref != nd]).sum())
