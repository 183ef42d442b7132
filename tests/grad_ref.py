"""FP64 CPU reference of the Horn slope loss and its adjoint (test helper).

Loss L(z) = sum_c (slope(z)(c) - slope(z_ref)(c))^2 over the cells where both
slopes exist (windows free of nodata, the ring excluded), slope as the
reference's Horn formula (apps/morphology/slope/slopeOperator.cpp:51-86).
``adjoint64`` is the hand-derived gradient in FP64; ``fd_errors`` compares it
with FP64 central finite differences of the loss, cell by cell.
"""
import numpy as np

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


def fd_errors(z, zr, cs, g64, cells, h=1e-4):
    """Relative error of g64 against FP64 central differences of the loss at
    each of `cells` (flat indices; nodata cells skipped), as
    |fd - g| / max(|g|, 1e-6 max|g64|).  Returns (errors, fd values, indices).
    fd is the Richardson combination (4 D(h/2) - D(h)) / 3 of the central
    differences D(s) = (L(z + s e) - L(z - s e)) / 2s with steps h and h/2
    metres: its truncation error is O(h^4), where a single central difference
    leaves O(h^2) -- ~5e-6 relative at h = 1e-3 m and ~3e-6 at 1e-4 m on cells
    of near-zero slope, against ~8e-8 for the combination at h = 1e-4 m.
    The loss is evaluated on a 7 x 7 patch around the cell: only the slopes of
    its 3 x 3 neighbourhood depend on z(cell)."""
    R, C = z.shape
    scale = float(np.abs(g64).max())
    z64 = z.astype(np.float64)
    zr64 = zr.astype(np.float64)
    errs, fds, idx = [], [], []
    for flat in cells:
        r, c = divmod(int(flat), C)
        if z[r, c] == ND:
            continue
        r0, r1, c0, c1 = max(r - 3, 0), min(r + 4, R), max(c - 3, 0), min(c + 4, C)
        patch = z64[r0:r1, c0:c1]
        _, _, sr, _ = horn64(zr64[r0:r1, c0:c1], cs)
        rr, cc = r - r0, c - c0
        sel = np.zeros(sr.shape, bool)
        sel[max(rr - 1, 1):rr + 2, max(cc - 1, 1):cc + 2] = True
        sel[0, :] = sel[-1, :] = sel[:, 0] = sel[:, -1] = False
        # a patch border that is not the raster's border is not a ring: the
        # cells selected above are at least one cell inside the patch, so their
        # windows lie inside it and their slopes are the full raster's
        def local(zz):
            _, _, s, _ = horn64(zz, cs)
            ok = ~np.isnan(s) & ~np.isnan(sr)
            return float(((s - sr)[ok & sel] ** 2).sum())
        def central(step):
            zp = patch.copy()
            zm = patch.copy()
            zp[rr, cc] += step
            zm[rr, cc] -= step
            return (local(zp) - local(zm)) / (2 * step)
        fd = (4.0 * central(h / 2) - central(h)) / 3.0
        ref = g64[r, c]
        errs.append(abs(fd - ref) / max(abs(ref), 1e-6 * scale))
        fds.append(fd)
        idx.append((r, c))
    return np.array(errs), np.array(fds), idx
