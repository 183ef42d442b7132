"""Hand-written adjoint of Horn slope on the GPU against an FP64 CPU adjoint
and FP64 central finite differences.

Loss L(z) = sum_c (slope(z)(c) - slope(z_ref)(c))^2 over cells where both
slopes exist.  Subgradient at zero slope: 0.  Tolerances (stated here):
the FP32 GPU gradient is compared normwise against the FP64 adjoint,
||g_gpu - g64||_inf <= 1e-4 ||g64||_inf, and the FP64 adjoint against FP64
central differences on 10^4 seeded cells, max relative error <= 1e-6.
"""
import numpy as np
import pytest

from gpu_helpers import dev, empty_dev, host
from pargo_gb300 import abi, synth

pytestmark = pytest.mark.gpu

ND = -9999.0


def horn64(z, cs):
    """FP64 Horn numerators and slope over the work rectangle; NaN where the
    window touches nodata (Eps 1e-7) or on the ring."""
    z = z.astype(np.float64)
    bad = np.abs(z - ND) < 1e-7
    R, C = z.shape
    nx = np.full((R, C), np.nan)
    ny = np.full((R, C), np.nan)
    w = lambda a, b: z[1 + a:R - 1 + a, 1 + b:C - 1 + b]
    nx[1:-1, 1:-1] = (w(-1, 1) - w(-1, -1)) + 2 * (w(0, 1) - w(0, -1)) + (w(1, 1) - w(1, -1))
    ny[1:-1, 1:-1] = (w(-1, -1) - w(1, -1)) + 2 * (w(-1, 0) - w(1, 0)) + (w(-1, 1) - w(1, 1))
    badw = np.zeros((R, C), bool)
    for a in (-1, 0, 1):
        for b in (-1, 0, 1):
            badw[1:-1, 1:-1] |= bad[1 + a:R - 1 + a, 1 + b:C - 1 + b]
    badw[0, :] = badw[-1, :] = badw[:, 0] = badw[:, -1] = True
    nx[badw] = np.nan
    ny[badw] = np.nan
    k = 1.0 / (8.0 * float(np.float32(cs)))
    return nx, ny, k * np.sqrt(nx * nx + ny * ny), k


def loss64(z, zr, cs):
    _, _, s, _ = horn64(z, cs)
    _, _, sr, _ = horn64(zr, cs)
    ok = ~np.isnan(s) & ~np.isnan(sr)
    return float(((s - sr)[ok] ** 2).sum())


def adjoint64(z, zr, cs):
    nx, ny, s, k = horn64(z, cs)
    _, _, sr, _ = horn64(zr, cs)
    ok = ~np.isnan(s) & ~np.isnan(sr)
    nn = np.sqrt(nx * nx + ny * ny)
    g = np.where(ok, 2 * (s - sr), 0.0)
    f = np.where(ok & (nn > 0), g * k / np.where(nn > 0, nn, 1), 0.0)
    A = np.nan_to_num(f * nx)
    B = np.nan_to_num(f * ny)
    a = [-1, 0, 1, -2, 0, 2, -1, 0, 1]
    b = [1, 2, 1, 0, 0, 0, -1, -2, -1]
    R, C = z.shape
    Ap = np.pad(A, 1)
    Bp = np.pad(B, 1)
    gz = np.zeros((R, C))
    for j in range(9):
        dr, dc = j // 3 - 1, j % 3 - 1
        # c = q - (dr, dc)
        gz += a[j] * Ap[1 - dr:1 - dr + R, 1 - dc:1 - dc + C] + b[j] * Bp[1 - dr:1 - dr + R, 1 - dc:1 - dc + C]
    return gz


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
    h = 1e-3
    worst = 0.0
    z64 = z.astype(np.float64)
    zr64 = zr.astype(np.float64)
    for idx in cells[:10000]:
        r, c = divmod(int(idx), C)
        if z[r, c] == ND:
            continue
        r0, r1, c0, c1 = max(r - 3, 0), min(r + 4, R), max(c - 3, 0), min(c + 4, C)
        zp = z64[r0:r1, c0:c1].copy()
        zm = zp.copy()
        zp[r - r0, c - c0] += h
        zm[r - r0, c - c0] -= h
        # local loss over the patch interior (cells whose window is inside the patch)
        def local(zz):
            _, _, s, _ = horn64(zz, cs)
            _, _, sr, _ = horn64(zr64[r0:r1, c0:c1], cs)
            ok = ~np.isnan(s) & ~np.isnan(sr)
            # keep only cells whose slope depends on (r, c) and is computed like in the full raster
            sel = np.zeros_like(ok)
            rr, cc = r - r0, c - c0
            sel[max(rr - 1, 1):rr + 2, max(cc - 1, 1):cc + 2] = True
            sel[0, :] = sel[-1, :] = sel[:, 0] = sel[:, -1] = False
            if r0 == 0:
                pass
            return float(((s - sr)[ok & sel] ** 2).sum())
        fd = (local(zp) - local(zm)) / (2 * h)
        ref = g64[r, c]
        denom = max(abs(ref), 1e-6 * scale)
        worst = max(worst, abs(fd - ref) / denom)
    assert worst <= 1e-3, worst


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
