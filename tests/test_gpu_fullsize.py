"""Parity at the full sizes of the benchmark workloads, through the C ABI.

* D8 + pit removal on the 8192^2 hydro DEM (seed 1, H 0.75, 0-3000 m, 30 m,
  1% pits, 10% nodata blob): the float64 levels bit for bit against the
  oracle's priority flood at gap 1e-3 and 5e-4, the float32 levels equal to
  those rounded, the D8 codes on the levels bit for bit.
* SCA on the filled 16384^2 DEM of the slope generator (seed 2, H 0.8,
  0-2000 m, 10 m cells): the levels proven equal to the reference's by the
  fixpoint equations (tests/fill_check.py), D8 bit for bit, both SCA
  contracts bit for bit against the oracle on those codes.
* Fused slope + D8 on the 32768^2 float32 DEM: D8 bit for bit, slope within
  1e-5 relative (plus the reference's own FP64 rounding floor), checked in
  bands of rows against the threaded FP64 oracle; max and mean relative error
  printed.
* Batched slope + D8 over all 512 uneven rasters (seeds 100-611): every
  raster's outputs against the oracle.
* Slope forward + adjoint on the 8192^2 DEM (seed 3): the FP32 gradient
  normwise within 1e-4 of the FP64 adjoint, the FP64 adjoint within 1e-6 of
  FP64 central differences on 10^4 seeded cells; max relative errors printed.

`pytest -s` shows the printed error figures.
"""
import os

import numpy as np
import pytest
import torch

from conftest import bits_equal
from fill_check import fill_fixpoint_mismatches
from gpu_helpers import d8_as_f64, dev, empty_dev, host, ref_noise_floor
from pargo_gb300 import abi, synth

pytestmark = pytest.mark.gpu

ND = -9999.0
THREADS = os.cpu_count() or 1


@pytest.mark.parametrize("gap", [1e-3, 5e-4])
def test_fill_and_d8_8192_bit_exact(gap, ctx, oracle_lib):
    dem = synth.hydro_dem(8192, 8192, seed=1, hurst=0.75, relief=3000.0)
    R = abi.raster
    d = dev(dem)
    w = empty_dev(dem.shape, np.float64)
    c = empty_dev(dem.shape, np.int8)
    st = ctx.hydro_pipeline(R(d, ND, 30.0), wdem=R(w, ND), d8=R(c, -128), gap=gap)
    W, codes = host(w), host(c)
    w32 = empty_dev(dem.shape, np.float32)
    ctx.fill(R(d, ND, 30.0), R(w32, ND), gap=gap)
    W32 = host(w32)
    del d, w, c, w32
    torch.cuda.empty_cache()
    ref = oracle_lib.fill(dem, ND, gap=gap)
    assert bits_equal(W, ref)
    assert np.array_equal(W32, ref.astype(np.float32))
    assert st.raised_cells == int((ref[ref != ND] > dem[ref != ND]).sum())
    assert st.raised_cells > 100000
    del W, W32
    d8ref = oracle_lib.d8(ref, ND, threads=THREADS)
    assert bits_equal(d8_as_f64(codes, -128), d8ref)


def test_sca_16384_both_contracts_bit_exact(ctx, oracle_lib):
    dem = synth.slope_dem(16384, 16384, seed=2, hurst=0.8, relief=2000.0)
    R = abi.raster
    d = dev(dem)
    w = empty_dev(dem.shape, np.float64)
    c = empty_dev(dem.shape, np.int8)
    ctx.hydro_pipeline(R(d, ND, 10.0), wdem=R(w, ND), d8=R(c, -128), gap=1e-3)
    del d
    W = host(w)
    del w
    torch.cuda.empty_cache()
    outs = {}
    for contract in (abi.SCA_CONVERGED, abi.SCA_SHIPPED):
        o = empty_dev(dem.shape, np.float64)
        ctx.sca(R(c, -128), R(o, ND), contract=contract)
        outs[contract] = host(o)
        del o
        torch.cuda.empty_cache()
    codes = host(c)
    del c
    torch.cuda.empty_cache()
    # the levels: the reference's fixpoint, proven cell by cell
    assert fill_fixpoint_mismatches(dem, W, ND, gap=1e-3) == 0
    assert (W > dem).sum() > 100000
    del dem
    d8ref = oracle_lib.d8(W, ND, threads=THREADS)
    del W
    assert bits_equal(d8_as_f64(codes, -128), d8ref)
    del codes
    conv, ship = oracle_lib.sca_both(d8ref, ND)
    assert bits_equal(outs[abi.SCA_CONVERGED], conv)
    assert bits_equal(outs[abi.SCA_SHIPPED], ship)


def test_slope_d8_32768_target(ctx, oracle_lib):
    side = 32768
    dem = synth.slope_dem(side, side, seed=0, hurst=0.8, relief=2000.0)
    R = abi.raster
    d = torch.from_numpy(dem).cuda()
    s = torch.empty((side, side), dtype=torch.float32, device="cuda")
    c = torch.empty((side, side), dtype=torch.int8, device="cuda")
    ctx.slope_d8(R(d, ND, 30.0), R(s, ND), R(c, -128))
    del d
    S, Cc = host(s), host(c)
    del s, c
    torch.cuda.empty_cache()
    atol = ref_noise_floor(dem, 30.0)
    band = 2048
    mx, rel_sum, rel_n, d8_bad, s_bad = 0.0, 0.0, 0, 0, 0
    for r0 in range(0, side, band):
        r1 = min(r0 + band, side)
        a0, a1 = max(r0 - 1, 0), min(r1 + 1, side)     # the band with a one-row halo
        sub = dem[a0:a1]
        sref = oracle_lib.slope(sub, ND, 30.0, threads=THREADS)[r0 - a0:r0 - a0 + (r1 - r0)]
        dref = oracle_lib.d8(sub, ND, threads=THREADS)[r0 - a0:r0 - a0 + (r1 - r0)]
        # a band's halo rows are nodata to the oracle: only the raster's first and
        # last rows are really the ring, and there both give nodata
        g = S[r0:r1].astype(np.float64)
        nd_r = sref == ND
        s_bad += int((nd_r != (g == ND)).sum())
        v = ~nd_r
        err = np.abs(g[v] - sref[v])
        scale = np.abs(sref[v])
        s_bad += int((err > 1e-5 * scale + atol).sum())
        big = scale > atol * 1e3
        rel = err[big] / scale[big]
        if rel.size:
            mx = max(mx, float(rel.max()))
            rel_sum += float(rel.sum())
            rel_n += rel.size
        d8_bad += int((d8_as_f64(Cc[r0:r1], -128) != dref).sum())
    print("32768^2 slope vs FP64 oracle: max rel %.3e, mean rel %.3e over %d cells; D8 mismatches %d"
          % (mx, rel_sum / max(rel_n, 1), rel_n, d8_bad))
    assert d8_bad == 0
    assert s_bad == 0


def test_batch512_every_raster_against_oracle(ctx, oracle_lib):
    shapes = synth.batch_shapes(512, first_seed=100)
    R = abi.raster
    dems, dd, ss, cc = [], [], [], []
    for (seed, r, c, h) in shapes:
        dem = synth.slope_dem(r, c, seed=seed, hurst=h, relief=2000.0)
        dems.append(dem)
        dd.append(dev(dem, 16))
        ss.append(empty_dev(dem.shape, np.float32, 16))
        cc.append(empty_dev(dem.shape, np.int8, 16))
    ctx.batch_slope_d8([R(x, ND, 30.0) for x in dd], [R(x, ND) for x in ss], [R(x, -128) for x in cc])
    torch.cuda.synchronize()
    mx, rel_sum, rel_n, bad = 0.0, 0.0, 0, []
    for k, dem in enumerate(dems):
        S, C = host(ss[k]).astype(np.float64), host(cc[k])
        if not bits_equal(d8_as_f64(C, -128), oracle_lib.d8(dem, ND, threads=THREADS)):
            bad.append((k, "d8"))
        sref = oracle_lib.slope(dem, ND, 30.0, threads=THREADS)
        v = sref != ND
        if not np.array_equal(S == ND, ~v):
            bad.append((k, "slope nodata"))
            continue
        err = np.abs(S[v] - sref[v])
        scale = np.abs(sref[v])
        if not (err <= 1e-5 * scale).all():
            bad.append((k, "slope"))
        rel = err[scale > 0] / scale[scale > 0]
        mx = max(mx, float(rel.max()))
        rel_sum += float(rel.sum())
        rel_n += rel.size
    print("batch512 (%d cells): slope max rel %.3e, mean rel %.3e; rasters off: %s"
          % (sum(d.size for d in dems), mx, rel_sum / max(rel_n, 1), bad))
    assert not bad


def test_gradient_8192_against_fp64_adjoint_and_finite_differences(ctx):
    from grad_ref import adjoint64, fd_errors, loss64
    side, cs = 8192, 30.0
    z = synth.slope_dem(side, side, seed=3, hurst=0.8, relief=2000.0)
    zr = synth.perturbed(z, sigma=0.5, seed=3)
    R = abi.raster
    gz = empty_dev(z.shape, np.float32)
    loss = ctx.slope_loss_grad(R(dev(z), ND, cs), R(dev(zr), ND, cs), R(gz, ND))
    g_gpu = host(gz)
    del gz
    torch.cuda.empty_cache()
    g64 = adjoint64(z, zr, cs)
    L64 = loss64(z, zr, cs)
    scale = float(np.abs(g64).max())
    norm_err = float(np.abs(g_gpu.astype(np.float64) - g64).max()) / scale
    rng = np.random.default_rng(3)
    cells = rng.integers(0, side * side, size=10000)
    errs, fds, idx = fd_errors(z, zr, cs, g64, cells, h=1e-4)
    gsel = np.array([g_gpu[r, c] for r, c in idx], np.float64)
    gpu_vs_fd = np.abs(gsel - fds) / np.maximum(np.abs(fds), 1e-6 * scale)
    print("8192^2 gradient: loss rel err %.3e; FP32 GPU vs FP64 adjoint normwise %.3e; FP64 adjoint vs FP64 "
          "central differences (10^4 cells) max rel %.3e; FP32 GPU vs central differences max rel %.3e"
          % (abs(loss - L64) / L64, norm_err, float(errs.max()), float(gpu_vs_fd.max())))
    assert abs(loss - L64) <= 1e-4 * L64
    assert norm_err <= 1e-4
    assert float(errs.max()) <= 1e-6
    assert float((np.abs(gsel - fds)).max()) <= 1e-4 * scale
