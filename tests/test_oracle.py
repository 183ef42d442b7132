"""Pins the CPU oracle (oracle/pargo_oracle.c) to the reference.

1. Against the committed golden fixtures, which the unmodified reference
   operators produced (tests/golden/make_golden.py): bit-exact, every case,
   every operator output.
2. Against the reference operators themselves (oracle/_ref), where the
   reference tree is present, on extra seeded inputs.
"""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, bits_equal, load_golden


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_oracle_matches_golden(case, oracle_lib):
    g = load_golden(case)
    dem, nd, cs = g["dem"], float(g["nodata"]), float(g["cellsize"])
    O = oracle_lib
    for m in range(7):
        assert bits_equal(O.slope(dem, nd, cs, method=m), g["slope_m%d" % m]), "slope method %d" % m
    assert bits_equal(O.d8(dem, nd, dir_type=8), g["d8_8"])
    assert bits_equal(O.d8(dem, nd, dir_type=256), g["d8_256"])
    w_gs, sweeps = O.fill_gs(dem, nd)
    assert bits_equal(w_gs, g["fill"])
    assert sweeps == int(g["fill_sweeps"])
    assert bits_equal(O.fill(dem, nd), g["fill"]), "priority-flood fixpoint differs from the reference sweeps"
    assert bits_equal(O.d8(g["fill"], nd, dir_type=8), g["d8w_8"])
    ship, _ = O.sca_sweeps(g["d8w_8"], nd, 1)
    assert bits_equal(ship, g["sca_ship"])
    conv, _ = O.sca_sweeps(g["d8w_8"], nd, 1 << 30)
    assert bits_equal(conv, g["sca_conv"])
    assert bits_equal(O.sca(g["d8w_8"], nd), g["sca_conv"])
    assert bits_equal(O.sca(g["d8w_8"], nd, shipped=True), g["sca_ship"])


def test_golden_fixture_facts():
    """Facts of dem.tif the reference itself printed when the fixtures were made."""
    g = load_golden("demtif")
    dem = g["dem"]
    assert dem.shape == (124, 104)
    assert float(g["cellsize"]) == 90.0
    assert int(g["fill_sweeps"]) == 25
    valid = g["slope_m0"] != -9999.0
    assert valid.sum() == 6806
    assert (g["fill"] > dem.astype(np.float64)).sum() > 0


def _ref():
    import oracle
    if not oracle.Reference.available():
        pytest.skip("reference tree absent: fixtures carry the reference results")
    return oracle.Reference()


@pytest.mark.parametrize("seed,shape", [(21, (57, 70)), (22, (33, 129)), (23, (120, 45))])
def test_oracle_matches_reference_binary(seed, shape, oracle_lib):
    from pargo_gb300 import synth
    R = _ref()
    O = oracle_lib
    dem = synth.hydro_dem(shape[0], shape[1], seed=seed, hurst=0.7, relief=800.0)
    nd, cs = -9999.0, 25.0
    for m in range(7):
        assert bits_equal(O.slope(dem, nd, cs, method=m), R.slope(dem, nd, cs, method=m))
    for dt in (8, 256):
        assert bits_equal(O.d8(dem, nd, dir_type=dt), R.d8(dem, nd, cs, dir_type=dt))
    w_ref, sw_ref = R.fill(dem, nd, cs)
    w_gs, sw = O.fill_gs(dem, nd)
    assert bits_equal(w_gs, w_ref) and sw == sw_ref
    assert bits_equal(O.fill(dem, nd), w_ref)
    d8w = R.d8(w_ref, nd, cs)
    assert bits_equal(O.d8(w_ref, nd), d8w)
    assert bits_equal(O.sca(d8w, nd), R.sca(d8w, nd, cs, converged=True)[0])
    assert bits_equal(O.sca(d8w, nd, shipped=True), R.sca(d8w, nd, cs, converged=False)[0])


def test_oracle_openmp_matches_serial(oracle_lib):
    """The threaded slope/D8 restatement (the CPU baseline) gives the serial bytes."""
    from pargo_gb300 import synth
    dem = synth.slope_dem(300, 257, seed=4)
    O = oracle_lib
    assert bits_equal(O.slope(dem, -9999.0, 30.0, threads=4), O.slope(dem, -9999.0, 30.0, threads=1))
    assert bits_equal(O.d8(dem, -9999.0, threads=4), O.d8(dem, -9999.0, threads=1))


def test_planted_mistake_is_caught(oracle_lib):
    """A wrong oracle must fail the golden comparison: plant an off-by-one-ulp
    change in the fixture's slope and in the fill, on the CPU."""
    g = load_golden("fbm_slope")
    s = oracle_lib.slope(g["dem"], -9999.0, 30.0)
    bad = s.copy()
    k = np.flatnonzero(bad != -9999.0)[10]
    bad.flat[k] = np.nextafter(bad.flat[k], np.inf)
    assert not bits_equal(bad, g["slope_m0"])
    h = load_golden("fbm_hydro")
    w = oracle_lib.fill(h["dem"], -9999.0, gap=0.0005 * (1 + 1e-9))
    assert not bits_equal(w, h["fill"])


@pytest.mark.parametrize("gap", [1e-3, 2.0 ** -10, 3 * 2.0 ** -12])
def test_oracle_fill_near_zero_levels(gap, oracle_lib):
    """Levels at and just above 0, where x + gap leaves x's binade or ties:
    the priority flood and the raster-order sweeps agree bit for bit."""
    from conftest import near_zero_dem
    dem = near_zero_dem(61, 77, seed=3)
    w_pf = oracle_lib.fill(dem, -9999.0, gap=gap)
    w_gs, _ = oracle_lib.fill_gs(dem, -9999.0, gap=gap)
    assert bits_equal(w_pf, w_gs)
    assert (w_pf > dem).sum() > 100


def test_oracle_fill_near_zero_matches_reference_binary(oracle_lib):
    from conftest import near_zero_dem
    R = _ref()
    dem = near_zero_dem(61, 77, seed=3)
    w_ref, sw_ref = R.fill(dem, -9999.0, 1.0)
    w_gs, sw = oracle_lib.fill_gs(dem, -9999.0)
    assert bits_equal(w_gs, w_ref) and sw == sw_ref
    assert bits_equal(oracle_lib.fill(dem, -9999.0), w_ref)


@pytest.mark.parametrize("seed,shape", [(31, (90, 120)), (32, (47, 203))])
def test_oracle_twi_matches_reference_binary(seed, shape, oracle_lib):
    """The TWI restatement against the reference TWIOperator, on a filled,
    routed DEM (nodata windows, flat cells where slope is raised to 1e-7)."""
    from pargo_gb300 import synth
    R = _ref()
    O = oracle_lib
    dem = synth.hydro_dem(shape[0], shape[1], seed=seed)
    w = O.fill(dem, -9999.0)
    sl = O.slope(w, -9999.0, 30.0)
    sca = O.sca(O.d8(w, -9999.0), -9999.0, shipped=True)
    sl[5, 5] = 0.0   # a zero slope: raised to Eps
    ref = R.twi(sl, sca, -9999.0, 30.0)
    assert bits_equal(O.twi(sl, sca, -9999.0), ref)
    assert (ref == -9999.0).any() and np.isfinite(ref).all()


@pytest.mark.parametrize("slp_exp", [-1.0, 0.0, 0.5, 1.0])
def test_oracle_mfd_matches_reference_binary(slp_exp, oracle_lib):
    """MFD-md weights (MFDOperator) and the MFD SCA (the scamfdmd operator's
    single accumulation sweep) against the reference built from its sources,
    bit for bit, on a filled DEM with nodata and flats; -1 is pMFDmd's default
    exponent."""
    from pargo_gb300 import synth
    R = _ref()
    if R.mfd_lib is None:
        pytest.skip("MFD-md reference build absent")
    O = oracle_lib
    dem = synth.hydro_dem(83, 117, seed=71, blob_fraction=0.05)
    w = O.fill(dem, -9999.0).astype(np.float32)
    w[40:44, 50:60] = w[40, 50]   # an exact flat
    a = O.mfd(w, -9999.0, 30.0, slp_exp)
    b = R.mfd(w, -9999.0, 30.0, slp_exp)
    assert bits_equal(a.reshape(8, -1), b.reshape(8, -1))
    assert bits_equal(O.sca_mfd(b, -9999.0), R.sca_mfd(b, -9999.0))


@pytest.mark.parametrize("shape,grain,ring,nparts,loads", [
    ((203, 157), 1, False, 5, (0.0, 1.0)),
    ((203, 157), 4, False, 7, (0.3, 1.7)),
    ((120, 333), 10, True, 3, (0.0, 1.0)),
    ((97, 61), 7, True, 9, (2.5, 0.25)),
    ((64, 64), 16, False, 2, (1.0, 1.0)),
    ((300, 40), 3, False, 90, (0.1, 3.0)),
])
def test_oracle_load_matches_reference_binary(shape, grain, ring, nparts, loads, oracle_lib):
    """The load estimator: the intensity-ratio compute layer (ComputeLayer +
    Transformation) bit for bit, the valRowDcmp cuts and getCompuLoad's data
    rows for rank 0, against the reference gpro classes on a DEM with a nodata
    blob and a nodata border."""
    from pargo_gb300 import synth
    R = _ref()
    dem = synth.hydro_dem(shape[0], shape[1], seed=shape[0] + grain, blob_fraction=0.2)
    dem[0, :] = -9999.0
    ref, comp, rank0 = R.compute_load(dem, -9999.0, grain, loads[0], loads[1], ring, nparts=nparts)
    got = oracle_lib.compute_load(dem, -9999.0, grain, loads[0], loads[1], ring)
    assert bits_equal(got, ref)
    oc, ob = oracle_lib.load_decompose(got, -9999.0, shape, nparts, ring)
    assert np.array_equal(oc, comp)
    assert np.array_equal(ob[0], rank0)
    # the parts tile the data work rectangle
    assert ob[0, 0] == 1 and ob[-1, 2] == shape[0] - 2
    assert all(ob[i + 1, 0] == ob[i, 2] + 1 for i in range(nparts - 1))
