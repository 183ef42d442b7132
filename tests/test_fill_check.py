"""The fixpoint check of tests/fill_check.py, pinned on the CPU: it accepts
the reference's own pit-removal results (golden fixtures) and the oracle's,
and it rejects surfaces with a planted mistake -- one level off by one ulp, a
surface that raised nothing, a relaxation stopped before its fixpoint."""
import numpy as np
import pytest

from conftest import GOLDEN_CASES, load_golden, near_zero_dem
from fill_check import fill_fixpoint_mismatches
from pargo_gb300 import synth


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_accepts_reference_results(case):
    g = load_golden(case)
    assert fill_fixpoint_mismatches(g["dem"], g["fill"], float(g["nodata"]), gap=0.0005) == 0


@pytest.mark.parametrize("gap", [1e-3, 5e-4, 3 * 2.0 ** -12])
def test_accepts_oracle_and_rejects_planted_mistakes(gap, oracle_lib):
    dem = synth.hydro_dem(300, 411, seed=31)
    w = oracle_lib.fill(dem, -9999.0, gap=gap)
    assert fill_fixpoint_mismatches(dem, w, gap=gap, band=64) == 0
    raised = np.argwhere(w > dem)
    assert len(raised) > 100
    r, c = raised[len(raised) // 2]
    off = w.copy()
    off[r, c] = np.nextafter(off[r, c], np.inf)           # one level one ulp high
    assert fill_fixpoint_mismatches(dem, off, gap=gap) > 0
    off[r, c] = np.nextafter(w[r, c], -np.inf)            # one ulp low
    assert fill_fixpoint_mismatches(dem, off, gap=gap) > 0
    flat = np.where(w == -9999.0, w, dem.astype(np.float64))   # raised nothing
    assert fill_fixpoint_mismatches(dem, flat, gap=gap) > 0


def test_rejects_an_unconverged_relaxation(oracle_lib):
    """A Gauss-Seidel relaxation stopped after a few sweeps is a surface no
    later check would catch by its range alone: the equations catch it."""
    import ctypes

    import oracle
    dem = synth.hydro_dem(200, 260, seed=33)
    O = oracle_lib
    out = np.empty(dem.shape, np.float64)
    sw = ctypes.c_int(0)
    a = np.ascontiguousarray(dem, np.float32)
    rc = O.lib.orc_fill_gs(a.ctypes.data_as(oracle._c_f32p), a.shape[0], a.shape[1], -9999.0, 1e-3, 10000.0, 4,
                           out.ctypes.data_as(oracle._c_f64p), ctypes.byref(sw))
    assert rc == 2                                         # stopped at its sweep cap
    assert fill_fixpoint_mismatches(dem, out, gap=1e-3) > 0
    assert fill_fixpoint_mismatches(dem, O.fill(dem, -9999.0, gap=1e-3), gap=1e-3) == 0


def test_near_zero_levels(oracle_lib):
    dem = near_zero_dem(96, 130, seed=7)
    for gap in (1e-3, 2.0 ** -10):
        w = oracle_lib.fill(dem, -9999.0, gap=gap)
        assert fill_fixpoint_mismatches(dem, w, gap=gap) == 0
