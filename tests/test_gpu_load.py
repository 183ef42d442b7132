"""The load estimator on the GPU (pargo_compute_load, pargo_load_decompose)
against the oracle, which is pinned bit for bit to the reference gpro
ComputeLayer / Transformation / DeComposition (tests/test_oracle.py).  The
compute layer must be bit-identical (sequential FP64 sums in the reference's
order); the decomposition's compute rows and data rectangles identical."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, bits_equal
from gpu_helpers import dev, empty_dev, host
from pargo_gb300 import _paths, abi, synth

pytestmark = pytest.mark.gpu
ND = -9999.0


def _dem(shape, seed):
    d = synth.hydro_dem(shape[0], shape[1], seed=seed, blob_fraction=0.2)
    d[0, :] = ND
    return d


@pytest.mark.parametrize("shape,grain,ring,loads", [((203, 157), 1, False, (0.0, 1.0)),
                                                    ((203, 157), 4, False, (0.3, 1.7)),
                                                    ((1200, 1333), 10, True, (0.0, 1.0)),
                                                    ((97, 61), 7, True, (2.5, 0.25)),
                                                    ((2048, 4100), 64, False, (0.1, 3.0))])
def test_compute_layer_bit_exact(shape, grain, ring, loads, ctx, oracle_lib):
    dem = _dem(shape, shape[1] + grain)
    ref = oracle_lib.compute_load(dem, ND, grain, loads[0], loads[1], ring)
    out = empty_dev(ref.shape, np.float64)
    ctx.compute_load(abi.raster(dev(dem), ND), abi.raster(out, ND), grain, loads[0], loads[1], ring)
    assert bits_equal(host(out), ref)


@pytest.mark.parametrize("shape,grain,ring,loads,nl,dt", [((1030, 1234), 16, False, (0.0, 1.0), 1, np.float32),
                                                          ((517, 700), 8, True, (2.0, 5.0), 2, np.float32),
                                                          ((300, 333), 32, True, (1.0, 4.0), 1, np.float32),
                                                          ((203, 157), 2, True, (0.0, 1.0), 1, np.float64),
                                                          ((35, 35), 32, False, (0.0, 1.0), 1, np.float32),
                                                          ((150, 190), 16, False, (3.0, 0.0), 2, np.float64)])
def test_integer_loads_counted_by_columns(shape, grain, ring, loads, nl, dt, ctx, oracle_lib):
    """Integer loads with a grain dividing 32 take the column-counting kernel
    (warps over 32 consecutive data columns): ragged last compute rows and
    columns, the compute ring, several layers, float32 and float64 data."""
    layers = [_dem(shape, 11 * k + grain).astype(dt) for k in range(nl)]
    ref = oracle_lib.compute_load(np.stack(layers) if nl > 1 else layers[0], ND, grain, loads[0], loads[1], ring)
    out = empty_dev(ref.shape, np.float64)
    ctx.compute_load([abi.raster(dev(x), ND) for x in layers], abi.raster(out, ND), grain, loads[0], loads[1], ring)
    assert bits_equal(host(out), ref)


def test_float64_data_several_layers_host_buffers(ctx, oracle_lib):
    a = _dem((150, 190), 5).astype(np.float64)
    b = _dem((150, 190), 6).astype(np.float64)
    ref = oracle_lib.compute_load(np.stack([a, b]), ND, 5, 0.5, 2.0)
    out = np.empty(ref.shape, np.float64)               # host in, host out
    ctx.compute_load([abi.raster(a, ND), abi.raster(b, ND)], abi.raster(out, ND), 5, 0.5, 2.0)
    assert bits_equal(out, ref)


@pytest.mark.parametrize("shape,grain,ring,nparts", [((203, 157), 1, False, 5), ((1200, 1333), 10, True, 8),
                                                     ((300, 40), 3, False, 90), ((97, 61), 7, True, 1),
                                                     ((4096, 512), 16, False, 152)])
def test_decomposition_matches_oracle(shape, grain, ring, nparts, ctx, oracle_lib):
    dem = _dem(shape, shape[0] + nparts)
    load = oracle_lib.compute_load(dem, ND, grain, 0.0, 1.0, ring)
    oc, ob = oracle_lib.load_decompose(load, ND, shape, nparts, ring)
    dl = dev(load)
    comp, bounds = ctx.load_decompose(abi.raster(dl, ND), shape, nparts, ring)
    assert np.array_equal(comp, oc) and np.array_equal(bounds, ob)
    comp2, bounds2 = ctx.load_decompose(abi.raster(load, ND), shape, nparts, ring)   # host compute layer
    assert np.array_equal(comp2, oc) and np.array_equal(bounds2, ob)


@pytest.mark.parametrize("loads,dt", [((0.3, 1.7), np.float64), ((0.0, 1.0), np.float32), ((0.25, 3.0), np.float32)])
def test_decomposition_of_fractional_and_float32_layers(loads, dt, ctx, oracle_lib):
    """Row loads summed in the reference's order where they are fractional
    (the warp's integer sum applies only to integer-valued rows), and from a
    float32 compute layer."""
    shape, grain, ring, nparts = (1200, 1333), 10, True, 8
    dem = _dem(shape, 31)
    load = oracle_lib.compute_load(dem, ND, grain, loads[0], loads[1], ring).astype(dt)
    oc, ob = oracle_lib.load_decompose(load.astype(np.float64), ND, shape, nparts, ring)
    comp, bounds = ctx.load_decompose(abi.raster(dev(load), ND), shape, nparts, ring)
    assert np.array_equal(comp, oc) and np.array_equal(bounds, ob)


def test_rejects_bad_arguments(ctx):
    dem = dev(_dem((50, 60), 1))
    cr, cc = abi.compute_load_dims(50, 60, 4)
    out = empty_dev((cr, cc), np.float64)
    for kw in (dict(grain=0), dict(grain=4, nodata_load=-1.0)):
        with pytest.raises(abi.PargoError):
            ctx.compute_load(abi.raster(dem, ND), abi.raster(out, ND), **kw)
    with pytest.raises(abi.PargoError):
        ctx.compute_load(abi.raster(dem, ND), abi.raster(empty_dev((cr + 1, cc), np.float64), ND), 4)
    with pytest.raises(abi.PargoError):
        ctx.load_decompose(abi.raster(out, ND), (50, 60), cr + 1)


def test_gpro_compute_layer_and_estimate_function(tmp_path, oracle_lib):
    """The gpro classes as the reference's reclassify / IDW mains use them:
    ComputeLayer::init + Transformation(nodataLoad, validLoad).run() +
    getCompuLoad, and an estimate-function subclass on the host."""
    from tiff_io import write_tiff
    dem = _dem((301, 257), 9)
    write_tiff(str(tmp_path / "dem.tif"), dem, ND, 30.0)
    (tmp_path / "moore.nbr").write_text("9\n0 0 1.0\n-1 -1 1.0\n-1 0 1.0\n-1 1 1.0\n0 -1 1.0\n0 1 1.0\n"
                                        "1 -1 1.0\n1 0 1.0\n1 1 1.0\n")
    exe = tmp_path / "load_selftest"
    inc = [os.path.join(ROOT, "pargo_gb300", "gpro", "include"), os.path.join(ROOT, "include")]
    subprocess.run(["g++", "-std=c++14", "-O1", "-Wall"] + ["-I" + d for d in inc] +
                   [os.path.join(ROOT, "tests", "cpp", "load_selftest.cpp"), "-o", str(exe),
                    "-L" + _paths.LIB_DIR, "-lpargo_gpro", "-lpargo_gpu", "-Wl,-rpath," + _paths.LIB_DIR], check=True)
    r = subprocess.run([str(exe), str(tmp_path / "dem.tif"), str(tmp_path / "moore.nbr"), "6", "6"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = dict(l.split(" ", 1) for l in r.stdout.strip().splitlines())
    load = oracle_lib.compute_load(dem, ND, 6, 0.0, 1.0)
    _, ob = oracle_lib.load_decompose(load, ND, dem.shape, 6)
    assert float(lines["sum"]) == float(load.sum())
    assert [int(v) for v in lines["rank0"].split()] == ob[0].tolist()
    assert [int(v) for v in lines["parts"].split()] == ob.ravel().tolist()
    est = np.arange(load.size, dtype=np.float64).reshape(load.shape) % 7     # the subclass's estimate
    _, eb = oracle_lib.load_decompose(est, ND, dem.shape, 6)
    assert [int(v) for v in lines["estimate_parts"].split()] == eb.ravel().tolist()
