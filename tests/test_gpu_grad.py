"""Hand-written adjoint of Horn slope on the GPU against an FP64 CPU adjoint
and FP64 central finite differences.

Loss L(z) = sum_c (slope(z)(c) - slope(z_ref)(c))^2 over cells where both
slopes exist.  Subgradient at zero slope: 0.  Tolerances (stated here):
the FP32 GPU gradient is compared normwise against the FP64 adjoint,
||g_gpu - g64||_inf <= 1e-4 ||g64||_inf, and the FP64 adjoint against FP64
central differences on 10^4 seeded cells, max relative error <= 1e-6
(|fd - g| / max(|g|, 1e-6 max|g|)).  The differences are Richardson-combined
central differences with steps 1e-4 and 5e-5 m (tests/grad_ref.py): a single
central difference carries an O(h^2) truncation error that alone reaches
~5e-6 at 1e-3 m on this surface; the combination measures below 1e-7.
"""
import numpy as np
import pytest

from gpu_helpers import dev, empty_dev, host
from grad_ref import adjoint64, fd_errors, loss64
from pargo_gb300 import abi, synth

pytestmark = pytest.mark.gpu

ND = -9999.0


def test_adjoint_against_fp64_and_finite_differences(ctx):
    R, C, cs = 384, 320, 30.0
    z = synth.slope_dem(R, C, seed=3, hurst=0.75, relief=3000.0)
    z[100:110, 50:60] = ND
    zr = synth.perturbed(z, seed=3, sigma=0.5)
    gz = empty_dev((R, C), np.float32)
    loss = ctx.slope_loss_grad(abi.raster(dev(z), ND, cs), abi.raster(dev(zr), ND, cs), abi.raster(gz, ND))
    g_gpu = host(gz).astype(np.float64)
    g64 = adjoint64(z, zr, cs)
    L64 = loss64(z, zr, cs)
    assert abs(loss - L64) <= 1e-4 * L64
    scale = np.abs(g64).max()
    assert np.abs(g_gpu - g64).max() <= 1e-4 * scale
    # FP64 central differences of the FP64 loss on 10^4 seeded cells
    rng = np.random.default_rng(3)
    cells = rng.integers(0, R * C, size=10000)
    errs, fds, idx = fd_errors(z, zr, cs, g64, cells, h=1e-4)
    worst = float(errs.max())
    print("adjoint vs FP64 central differences, %dx%d, %d cells: max rel %.3e" % (R, C, len(errs), worst))
    assert worst <= 1e-6, worst


def test_backward_only_matches_fused(ctx):
    R, C, cs = 200, 260, 10.0
    z = synth.slope_dem(R, C, seed=8)
    zr = synth.perturbed(z, seed=8, sigma=0.5)
    gz = empty_dev((R, C), np.float32)
    ctx.slope_loss_grad(abi.raster(dev(z), ND, cs), abi.raster(dev(zr), ND, cs), abi.raster(gz, ND), want_loss=False)
    s = empty_dev((R, C), np.float32)
    sr = empty_dev((R, C), np.float32)
    ctx.slope_fwd(abi.raster(dev(z), ND, cs), abi.raster(s, ND))
    ctx.slope_fwd(abi.raster(dev(zr), ND, cs), abi.raster(sr, ND))
    S, SR = host(s), host(sr)
    gs = np.where((S != ND) & (SR != ND), 2 * (S - SR), 0.0).astype(np.float32)
    gz2 = empty_dev((R, C), np.float32)
    ctx.slope_bwd(abi.raster(dev(z), ND, cs), abi.raster(dev(gs), ND), abi.raster(gz2, ND))
    a, b = host(gz).astype(np.float64), host(gz2).astype(np.float64)
    assert np.abs(a - b).max() <= 1e-5 * max(np.abs(a).max(), 1e-30)
