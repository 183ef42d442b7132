"""End to end through the gpro-compatible C++ layer and the application
mains: the reference's three-executable hydrology chain (pit removal ->
D8 -> SCA, through GeoTIFF files) and slope, on the reference's own dem.tif
data, compared with what the reference operators output (golden fixtures)."""
import os
import subprocess

import numpy as np
import pytest

from conftest import bits_equal, load_golden
from gpu_helpers import ref_noise_floor, slope_close
from pargo_gb300 import _paths
from tiff_io import read_tiff, write_tiff

pytestmark = pytest.mark.gpu

MOORE = "9\n0 0 1.0\n-1 -1 1.0\n-1 0 1.0\n-1 1 1.0\n0 -1 1.0\n0 1 1.0\n1 -1 1.0\n1 0 1.0\n1 1 1.0\n"


def run(app, *args, env=None):
    r = subprocess.run([os.path.join(_paths.BIN_DIR, app)] + [str(a) for a in args], capture_output=True, text=True,
                       env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "run time is" in r.stdout


@pytest.mark.parametrize("case", ["demtif", "fbm_hydro", "quantised"])
def test_app_chain_matches_reference(case, tmp_path):
    g = load_golden(case)
    nd, cs = float(g["nodata"]), float(g["cellsize"])
    nbr = tmp_path / "moore.nbr"
    nbr.write_text(MOORE)
    dem = tmp_path / "dem.tif"
    write_tiff(str(dem), g["dem"], nd, cs)
    run("pargo_pitremove", "-elev", dem, "-nbr", nbr, "-out", tmp_path / "fill.tif")
    w, wnd, _ = read_tiff(str(tmp_path / "fill.tif"))
    assert w.dtype == np.float64 and wnd == nd
    assert bits_equal(w, g["fill"])
    run("pargo_d8", tmp_path / "fill.tif", nbr, tmp_path / "d8.tif", 8)
    d8, _, _ = read_tiff(str(tmp_path / "d8.tif"))
    assert bits_equal(d8, g["d8w_8"])
    run("pargo_sca", tmp_path / "d8.tif", nbr, tmp_path / "sca.tif")
    sca, _, _ = read_tiff(str(tmp_path / "sca.tif"))
    assert bits_equal(sca, g["sca_ship"])  # the reference operator as shipped
    run("pargo_sca", tmp_path / "d8.tif", nbr, tmp_path / "sca_c.tif", "converged")
    sca_c, _, _ = read_tiff(str(tmp_path / "sca_c.tif"))
    assert bits_equal(sca_c, g["sca_conv"])
    for m, name in enumerate(["FD", "FFD", "MD", "SD", "SFD", "TFD", "TFDW"]):
        run("pargo_slope", "-elev", dem, "-nbr", nbr, "-slp", tmp_path / "s.tif", "-mtd", name)
        s, _, _ = read_tiff(str(tmp_path / "s.tif"))
        ok, mx, _ = slope_close(s, g["slope_m%d" % m], nd, atol=ref_noise_floor(g["dem"], cs))
        assert ok, (name, mx)
    run("pargo_d8", "-elev", dem, "-nbr", nbr, "-out", tmp_path / "d8r.tif", "-dirtype", 256)
    d8r, _, _ = read_tiff(str(tmp_path / "d8r.tif"))
    assert bits_equal(d8r, g["d8_256"])


@pytest.mark.parametrize("case", ["demtif", "fbm_hydro"])
def test_app_twi_after_the_chain(case, tmp_path, oracle_lib):
    """pTWI's step on the chain's files: slope of the filled DEM and the
    shipped SCA in, TWI out, against the oracle (pinned to TWIOperator) within
    the FP32 tolerance 1e-6 relative + 1e-6."""
    g = load_golden(case)
    nd, cs = float(g["nodata"]), float(g["cellsize"])
    nbr = tmp_path / "moore.nbr"
    nbr.write_text(MOORE)
    write_tiff(str(tmp_path / "fill.tif"), g["fill"], nd, cs)
    write_tiff(str(tmp_path / "sca.tif"), g["sca_ship"], nd, cs)
    run("pargo_slope", "-elev", tmp_path / "fill.tif", "-nbr", nbr, "-slp", tmp_path / "slope.tif")
    sl, _, _ = read_tiff(str(tmp_path / "slope.tif"))
    run("pargo_twi", tmp_path / "slope.tif", tmp_path / "sca.tif", nbr, tmp_path / "twi.tif")
    t, tnd, _ = read_tiff(str(tmp_path / "twi.tif"))
    ref = oracle_lib.twi(sl, g["sca_ship"], nd)
    assert tnd == nd and np.array_equal(t == nd, ref == nd)
    ok = ref != nd
    assert (np.abs(t[ok] - ref[ok]) <= 1e-6 * np.abs(ref[ok]) + 1e-6).all()


@pytest.mark.parametrize("case", ["demtif", "fbm_hydro"])
def test_app_mfd_then_sca_mfd(case, tmp_path, oracle_lib):
    """pMFDmd's and scamfdmd's steps on the filled DEM: the 8 weight files
    against the oracle (pinned to MFDOperator) within 1e-5 relative + 1e-6,
    then the MFD SCA of those files bit for bit against the oracle's sweep."""
    g = load_golden(case)
    nd, cs = float(g["nodata"]), float(g["cellsize"])
    nbr = tmp_path / "moore.nbr"
    nbr.write_text(MOORE)
    write_tiff(str(tmp_path / "fill.tif"), g["fill"], nd, cs)
    prefix = str(tmp_path / "mfd_")
    run("pargo_mfd", "-elev", tmp_path / "fill.tif", "-nbr", nbr, "-out", prefix, "-exp", 1.1)
    files = [prefix + "weightLayer%d.tif" % (i if i < 4 else i + 1) for i in range(8)]
    w = np.stack([read_tiff(f)[0] for f in files]).astype(np.float64)
    ref = oracle_lib.mfd(g["fill"], nd, cs, 1.1)
    assert np.array_equal(w == nd, ref == nd) and np.array_equal(w == 0, ref == 0)
    ok = ref != nd
    assert (np.abs(w[ok] - ref[ok]) <= 1e-5 * np.abs(ref[ok]) + 1e-6).all()
    run("pargo_sca_mfd", ",".join(files), nbr, tmp_path / "sca.tif")
    sca, snd, _ = read_tiff(str(tmp_path / "sca.tif"))
    assert snd == nd and bits_equal(sca, oracle_lib.sca_mfd(w, nd))


def test_app_rejects_bad_neighbourhood(tmp_path):
    g = load_golden("fbm_slope")
    dem = tmp_path / "dem.tif"
    write_tiff(str(dem), g["dem"], -9999.0, 30.0)
    nbr = tmp_path / "local.nbr"
    nbr.write_text("1\n0 0 1.0\n")
    r = subprocess.run([os.path.join(_paths.BIN_DIR, "pargo_slope"), dem, nbr, tmp_path / "s.tif"],
                       capture_output=True, text=True)
    assert r.returncode != 0
    assert "neighbourhood" in r.stderr
