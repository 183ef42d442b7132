"""Helpers shared by the GPU tests (device buffers through torch, raster views)."""
import numpy as np
import torch

from pargo_gb300 import abi

SLOPE_RTOL = 1e-5  # FP32 slope vs the reference's FP64 slope, relative, per cell


def dev(a, pitch_align=0):
    """Copy a numpy array to the GPU.  pitch_align > 0 pads each row to a
    multiple of that many bytes and returns a view of the valid columns."""
    t = torch.from_numpy(np.ascontiguousarray(a))
    if pitch_align:
        es = t.element_size()
        cols = a.shape[1]
        padded = (cols * es + pitch_align - 1) // pitch_align * pitch_align // es
        buf = torch.zeros((a.shape[0], padded), dtype=t.dtype, device="cuda")
        buf[:, :cols] = t.cuda()
        return buf[:, :cols]
    return t.cuda()


def empty_dev(shape, dtype, pitch_align=0):
    dt = {np.float32: torch.float32, np.float64: torch.float64, np.int8: torch.int8, np.int16: torch.int16,
          np.int32: torch.int32}[dtype]
    if pitch_align:
        es = torch.empty((), dtype=dt).element_size()
        padded = (shape[1] * es + pitch_align - 1) // pitch_align * pitch_align // es
        return torch.full((shape[0], padded), 77, dtype=dt, device="cuda")[:, :shape[1]]
    return torch.full(shape, 77, dtype=dt, device="cuda")


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def ref_noise_floor(dem, cellsize):
    """Absolute rounding bound of the reference's own FP64 slope: it sums raw
    elevations (slopeOperator.cpp:84-136), so where the exact answer is ~0 its
    result is rounding residue of order 2^-52 * (sum of |weights * elevations|)
    / (denominator * cellsize).  The weights of every method sum to <= 8 in
    magnitude, the denominators are >= 1; 2^-48 leaves a 16x margin."""
    z = np.asarray(dem, np.float64)
    v = z[np.isfinite(z) & (z != -9999.0)]
    zmax = float(np.abs(v).max()) if v.size else 0.0
    return 2.0 ** -48 * 8.0 * zmax / float(np.float32(cellsize))


def slope_close(gpu, ref, nodata=-9999.0, rtol=SLOPE_RTOL, atol=0.0):
    """Same nodata cells; |gpu - ref| <= rtol |ref| + atol on the others, where
    atol is the reference's own rounding floor (ref_noise_floor).  Returns
    (ok, max_rel, mean_rel) with the relative error taken over cells whose
    reference value is above atol."""
    gpu = np.asarray(gpu, np.float64)
    ref = np.asarray(ref, np.float64)
    nd_g = gpu == nodata
    nd_r = ref == nodata
    if not np.array_equal(nd_g, nd_r):
        return False, np.inf, np.inf
    v = ~nd_r
    if not v.any():
        return True, 0.0, 0.0
    err = np.abs(gpu[v] - ref[v])
    scale = np.abs(ref[v])
    ok = bool((err <= rtol * scale + atol).all())
    big = scale > max(atol, 0.0) * 1e3 if atol > 0 else scale > 0
    rel = err[big] / scale[big] if big.any() else np.zeros(1)
    return ok, float(rel.max()), float(rel.mean())


def d8_as_f64(codes, nodata_in, nodata_out=-9999.0):
    c = np.asarray(codes).astype(np.float64)
    c[np.asarray(codes) == nodata_in] = nodata_out
    return c
