"""The gpro-compatible C++ host layer (pargo_gb300/gpro), host-only parts:
GeoTIFF I/O, neighbourhoods, layer semantics; and that the reference's own
unmodified application mains compile and link against it (the drop-in)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from pargo_gb300 import _paths

INC = [os.path.join(ROOT, "pargo_gb300", "gpro", "include"), os.path.join(ROOT, "include")]
REF = os.environ.get("PARGO_REFERENCE_ROOT", "/root/reference")


def _link_args():
    return ["-L" + _paths.LIB_DIR, "-lpargo_gpro", "-lpargo_gpu", "-Wl,-rpath," + _paths.LIB_DIR]


def test_apps_are_built():
    for app in ("pargo_slope", "pargo_d8", "pargo_pitremove", "pargo_sca", "pargo_twi", "pargo_mfd", "pargo_sca_mfd"):
        assert os.access(os.path.join(_paths.BIN_DIR, app), os.X_OK), app
    assert os.path.exists(_paths.GPRO_SO)


def test_gpro_selftest(tmp_path):
    exe = tmp_path / "selftest"
    cmd = ["g++", "-std=c++14", "-O1", "-Wall"] + ["-I" + d for d in INC] + \
          [os.path.join(ROOT, "tests", "cpp", "gpro_selftest.cpp"), "-o", str(exe)] + _link_args()
    subprocess.run(cmd, check=True)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stderr


def test_load_estimator_classes_compile(tmp_path):
    """The gpro ComputeLayer / Transformation / DeComposition headers with an
    estimate-function subclass (tests/cpp/load_selftest.cpp) build and link."""
    exe = tmp_path / "load_selftest"
    cmd = ["g++", "-std=c++14", "-O1", "-Wall"] + ["-I" + d for d in INC] + \
          [os.path.join(ROOT, "tests", "cpp", "load_selftest.cpp"), "-o", str(exe)] + _link_args()
    subprocess.run(cmd, check=True)
    assert os.access(exe, os.X_OK)


def test_tiff_written_by_python_reads_in_cpp_and_back(tmp_path):
    from tiff_io import read_tiff, write_tiff
    a = (np.arange(60, dtype=np.float32).reshape(6, 10) * 1.5 - 7).astype(np.float32)
    a[2, 3] = -9999.0
    write_tiff(str(tmp_path / "p.tif"), a, -9999.0, 25.0)
    b, nd, cs = read_tiff(str(tmp_path / "p.tif"))
    assert np.array_equal(a, b) and nd == -9999.0 and cs == 25.0
    d = a.astype(np.float64) + 1e-9          # float64 stays float64
    write_tiff(str(tmp_path / "d.tif"), d, -9999.0, 25.0)
    e, _, _ = read_tiff(str(tmp_path / "d.tif"))
    assert e.dtype == np.float64 and np.array_equal(d, e)


@pytest.mark.parametrize("main", ["apps/morphology/slope/pSlope.cpp", "apps/hydrology/flowdird8/pD8.cpp",
                                  "apps/hydrology/pitremove/pPitRemove.cpp", "apps/hydrology/scad8/pSCA.cpp",
                                  "apps/hydrology/twi/pTWI.cpp", "apps/hydrology/flowdirmfdmd/pMFDmd.cpp",
                                  "apps/hydrology/scamfdmd/pSCA.cpp"])
def test_reference_main_compiles_against_gpu_gpro(main, tmp_path):
    """The reference's application main, byte for byte, built against the GPU
    gpro headers (copied to a scratch directory so that its quoted includes of
    the operator header resolve to the GPU operator, as a GPU build of the
    application would)."""
    src = os.path.join(REF, main)
    if not os.path.exists(src):
        pytest.skip("reference tree absent")
    local = tmp_path / os.path.basename(main)
    shutil.copyfile(src, local)
    exe = tmp_path / "main"
    cmd = ["g++", "-std=c++14", "-O1", "-w"] + ["-I" + d for d in INC] + [str(local), "-o", str(exe)] + _link_args()
    subprocess.run(cmd, check=True)
    assert os.access(exe, os.X_OK)
