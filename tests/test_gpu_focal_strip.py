"""The strip-walk form of fused slope + D8 (kernel variant "strip": warp-private
TMA pipelines down 128-cell column strips, deferred general-path rows),
forced through PARGO_FOCAL_VARIANT, against the reference's golden outputs
and the oracle, and bit for bit against the tiled kernel.  D8 must be
bit-exact; slope within 1e-5 relative."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, bits_equal, load_golden
from gpu_helpers import d8_as_f64, dev, empty_dev, host, ref_noise_floor, slope_close
from pargo_gb300 import abi, synth

pytestmark = pytest.mark.gpu
ND = -9999.0
STRIP = "5"      # the strip walk's variant index (after the five tiled variants)


@pytest.fixture
def strip(monkeypatch):
    monkeypatch.setenv("PARGO_FOCAL_VARIANT", STRIP)
    yield
    monkeypatch.delenv("PARGO_FOCAL_VARIANT", raising=False)


def _run(ctx, dem, cs=30.0, slope=True, d8=True):
    """Slope (float32) and/or D8 (int8) with 16-byte aligned rows, so the
    strip walk's vector stores apply."""
    R = abi.raster
    d = R(dev(dem, 16), ND, cs)
    s = empty_dev(dem.shape, np.float32, 16) if slope else None
    c = empty_dev(dem.shape, np.int8, 16) if d8 else None
    if slope and d8:
        ctx.slope_d8(d, R(s, ND), R(c, -128))
    elif slope:
        ctx.slope(d, R(s, ND))
    else:
        ctx.d8(d, R(c, -128))
    return (host(s) if slope else None), (host(c) if d8 else None)


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_strip_golden(case, ctx, strip):
    g = load_golden(case)
    nd, cs = float(g["nodata"]), float(g["cellsize"])
    s, c = _run(ctx, g["dem"], cs)
    ok, mx, _ = slope_close(s, g["slope_m0"], nd, atol=ref_noise_floor(g["dem"], cs))
    assert ok, mx
    assert bits_equal(d8_as_f64(c, -128, nd), g["d8_8"])


@pytest.mark.parametrize("shape", [(3, 3), (4, 5), (47, 127), (48, 128), (49, 129), (50, 131), (97, 385),
                                   (143, 257), (1024, 1024), (1500, 700)])
def test_strip_sizes_against_oracle(shape, ctx, oracle_lib, strip):
    """Segment (48 rows), stage (6 rows) and strip (128 columns) boundaries +-1."""
    dem = synth.hydro_dem(shape[0], shape[1], seed=shape[0] * 7 + shape[1], relief=1500.0)
    s, c = _run(ctx, dem)
    ok, mx, _ = slope_close(s, oracle_lib.slope(dem, ND, 30.0), ND)
    assert ok, mx
    assert bits_equal(d8_as_f64(c, -128, ND), oracle_lib.d8(dem, ND))


def test_strip_matches_tiled_bit_for_bit(ctx, monkeypatch):
    dem = synth.hydro_dem(2048, 1800, seed=41)
    monkeypatch.setenv("PARGO_FOCAL_VARIANT", "0")
    s0, c0 = _run(ctx, dem)
    monkeypatch.setenv("PARGO_FOCAL_VARIANT", STRIP)
    s1, c1 = _run(ctx, dem)
    assert np.array_equal(s0.view(np.int32), s1.view(np.int32))
    assert np.array_equal(c0, c1)


def test_strip_single_outputs_and_ties(ctx, oracle_lib, strip):
    rng = np.random.default_rng(5)
    q = rng.integers(0, 4, size=(300, 260)).astype(np.float32)   # exact ties everywhere
    _, c = _run(ctx, q, slope=False)
    assert bits_equal(d8_as_f64(c, -128, ND), oracle_lib.d8(q, ND))
    dem = synth.slope_dem(200, 333, seed=4)
    s, _ = _run(ctx, dem, d8=False)
    ok, mx, _ = slope_close(s, oracle_lib.slope(dem, ND, 30.0), ND)
    assert ok, mx


def test_strip_nodata_and_flat(ctx, strip):
    dem = np.full((60, 300), ND, np.float32)
    s, c = _run(ctx, dem)
    assert (s == ND).all() and (c == -128).all()
    flat = np.full((60, 300), 12.5, np.float32)
    s, c = _run(ctx, flat)
    assert (s[1:-1, 1:-1] == 0.0).all() and (c[1:-1, 1:-1] == -1).all()
    assert (s[0] == ND).all() and (c[:, -1] == -128).all()
