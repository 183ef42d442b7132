"""ctypes binding of the C ABI in ``include/pargo_gpu.h`` (``lib/libpargo_gpu.so``).

This is plumbing for Python callers, tests and the benchmark: every call goes
straight to the C entry point.  Rasters can be numpy arrays (host buffers,
staged by the library) or torch tensors (device buffers used in place).  The
library must be built; importing this module without it raises
``NativeLibraryMissing`` -- there is no Python or CPU fallback.
"""
import ctypes

import numpy as np

from . import _paths

PARGO_OK = 0
STATUS_NAMES = {
    0: "PARGO_OK", 1: "PARGO_ERR_INVALID_ARG", 2: "PARGO_ERR_NBR_UNSUPPORTED", 3: "PARGO_ERR_NOT_CONVERGED",
    4: "PARGO_ERR_CYCLE", 5: "PARGO_ERR_CUDA", 6: "PARGO_ERR_NO_DEVICE", 7: "PARGO_ERR_OUT_OF_MEMORY",
    8: "PARGO_ERR_DEVICE_TIMEOUT",
}
F32, F64, I8, I16, I32 = 0, 1, 2, 3, 4
HOST, DEVICE = 0, 1
SLOPE_FD, SLOPE_FFD, SLOPE_MD, SLOPE_SD, SLOPE_SFD, SLOPE_TFD, SLOPE_TFDW = range(7)
RATIO, DEGREES = 0, 1
SCA_CONVERGED, SCA_SHIPPED = 0, 1

_NP_DTYPES = {np.dtype(np.float32): F32, np.dtype(np.float64): F64, np.dtype(np.int8): I8,
              np.dtype(np.int16): I16, np.dtype(np.int32): I32}


class PargoError(RuntimeError):
    def __init__(self, status, message):
        self.status = status
        self.status_name = STATUS_NAMES.get(status, str(status))
        super().__init__("%s: %s" % (self.status_name, message))


class Raster(ctypes.Structure):
    _fields_ = [("data", ctypes.c_void_p), ("dtype", ctypes.c_int32), ("location", ctypes.c_int32),
                ("rows", ctypes.c_int64), ("cols", ctypes.c_int64), ("pitch", ctypes.c_int64),
                ("nodata", ctypes.c_double), ("cellsize", ctypes.c_double)]


class Nbr(ctypes.Structure):
    _fields_ = [("count", ctypes.c_int32), ("min_row", ctypes.c_int32), ("min_col", ctypes.c_int32),
                ("max_row", ctypes.c_int32), ("max_col", ctypes.c_int32)]


class FillOpts(ctypes.Structure):
    _fields_ = [("gap", ctypes.c_double), ("init_level", ctypes.c_double), ("max_rounds", ctypes.c_int64)]


class BatchOpts(ctypes.Structure):
    _fields_ = [("nodata_load", ctypes.c_double), ("valid_load", ctypes.c_double), ("order", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


BATCH_BY_INTENSITY, BATCH_BY_SIZE = 0, 1


class FillStats(ctypes.Structure):
    _fields_ = [("rounds", ctypes.c_int64), ("active_rounds", ctypes.c_int64), ("tile_visits", ctypes.c_int64),
                ("local_iterations", ctypes.c_int64), ("raised_cells", ctypes.c_int64), ("rounds_ms", ctypes.c_double)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(_paths.require(_paths.GPU_SO))
        P = ctypes.POINTER
        vp, i, st = ctypes.c_void_p, ctypes.c_int, ctypes.c_int
        R = P(Raster)
        N = P(Nbr)
        L.pargo_create.argtypes = [i, P(vp)]
        L.pargo_destroy.argtypes = [vp]
        L.pargo_last_error.argtypes = [vp]
        L.pargo_last_error.restype = ctypes.c_char_p
        L.pargo_abi_version.restype = i
        L.pargo_nbr_parse.argtypes = [ctypes.c_char_p, N]
        L.pargo_slope.argtypes = [vp, R, R, N, i, i, vp]
        L.pargo_d8.argtypes = [vp, R, R, N, i, vp]
        L.pargo_slope_d8.argtypes = [vp, R, R, R, N, i, i, i, vp]
        L.pargo_fill.argtypes = [vp, R, R, N, P(FillOpts), P(FillStats), vp]
        L.pargo_sca.argtypes = [vp, R, R, N, i, vp]
        L.pargo_twi.argtypes = [vp, R, R, R, N, vp]
        L.pargo_mfd.argtypes = [vp, R, R, N, ctypes.c_double, vp]
        L.pargo_sca_mfd.argtypes = [vp, R, R, N, vp]
        i64, i64p = ctypes.c_int64, P(ctypes.c_int64)
        L.pargo_compute_load_dims.argtypes = [i64, i64, i, i64p, i64p]
        L.pargo_compute_load.argtypes = [vp, i, R, N, i, i, ctypes.c_double, ctypes.c_double, R, vp]
        L.pargo_load_decompose.argtypes = [vp, R, i, i64, i64, N, i, i64p, i64p, vp]
        L.pargo_hydro_pipeline.argtypes = [vp, R, R, R, R, R, N, P(FillOpts), i, i, i, P(FillStats), vp]
        L.pargo_batch_slope_d8.argtypes = [vp, i, R, R, R, N, i, i, i, vp]
        L.pargo_batch_fill.argtypes = [vp, i, R, R, N, P(FillOpts), P(FillStats), vp]
        L.pargo_batch_slope_d8_ex.argtypes = [vp, i, R, R, R, N, i, i, i, P(BatchOpts), vp]
        L.pargo_batch_queue.argtypes = [vp, i, R, P(BatchOpts), ctypes.c_int64, P(ctypes.c_int64),
                                        P(ctypes.c_int32), P(ctypes.c_int64), P(ctypes.c_double), vp]
        L.pargo_slope_fwd.argtypes = [vp, R, R, N, vp]
        L.pargo_slope_bwd.argtypes = [vp, R, R, R, N, vp]
        L.pargo_slope_loss_grad.argtypes = [vp, R, R, R, P(ctypes.c_double), N, vp]
        L.pargo_sca_noalloc.argtypes = [R, R, N, i, vp]
        L.pargo_sca_noalloc.restype = st
        L.pargo_tune_focal.argtypes = [vp, R, i, P(i), P(ctypes.c_float), i]
        L.pargo_tune_focal.restype = st
        L.pargo_focal_num_variants.restype = i
        L.pargo_focal_variant_name.argtypes = [i]
        L.pargo_focal_variant_name.restype = ctypes.c_char_p
        L.pargo_focal_variant.argtypes = [vp, ctypes.c_int64]
        L.pargo_focal_variant.restype = i
        L.pargo_last_d8_fallbacks.argtypes = [vp]
        L.pargo_last_d8_fallbacks.restype = ctypes.c_int64
        for name in ("pargo_create", "pargo_destroy", "pargo_nbr_parse", "pargo_slope", "pargo_d8", "pargo_slope_d8",
                     "pargo_fill", "pargo_sca", "pargo_twi", "pargo_mfd", "pargo_sca_mfd", "pargo_compute_load_dims",
                     "pargo_compute_load", "pargo_load_decompose",
                     "pargo_hydro_pipeline", "pargo_batch_slope_d8", "pargo_batch_fill", "pargo_batch_slope_d8_ex",
                     "pargo_batch_queue", "pargo_slope_fwd",
                     "pargo_slope_bwd",
                     "pargo_slope_loss_grad"):
            getattr(L, name).restype = st
        _lib = L
    return _lib


def focal_variant_names():
    """Names of the fused slope+D8 kernel variants, by index."""
    L = lib()
    return [L.pargo_focal_variant_name(v).decode() for v in range(L.pargo_focal_num_variants())]


def compute_load_dims(rows, cols, grain):
    """Shape of the compute layer of a rows x cols raster at `grain`."""
    cr, cc = ctypes.c_int64(), ctypes.c_int64()
    rc = lib().pargo_compute_load_dims(rows, cols, grain, ctypes.byref(cr), ctypes.byref(cc))
    if rc:
        raise PargoError(rc, "bad compute layer arguments")
    return cr.value, cc.value


def nbr_parse(text):
    n = Nbr()
    rc = lib().pargo_nbr_parse(text.encode() if isinstance(text, str) else text, ctypes.byref(n))
    if rc:
        raise PargoError(rc, "invalid neighbourhood text")
    return n


MOORE = "9\n0 0 1.0\n-1 -1 1.0\n-1 0 1.0\n-1 1 1.0\n0 -1 1.0\n0 1 1.0\n1 -1 1.0\n1 0 1.0\n1 1 1.0\n"


def raster(a, nodata=-9999.0, cellsize=1.0):
    """Describe a 2-D numpy array (host) or torch tensor (its own device) as a
    pargo_raster.  The array must stay alive while the raster is in use."""
    try:
        import torch
        is_t = isinstance(a, torch.Tensor)
    except ImportError:  # pragma: no cover
        is_t = False
    if is_t:
        if a.dim() != 2 or a.stride(1) != 1:
            raise ValueError("raster tensors must be 2-D with unit column stride")
        dt = {"torch.float32": F32, "torch.float64": F64, "torch.int8": I8, "torch.int16": I16,
              "torch.int32": I32}[str(a.dtype)]
        loc = DEVICE if a.is_cuda else HOST
        r = Raster(a.data_ptr(), dt, loc, a.shape[0], a.shape[1], a.stride(0) * a.element_size(),
                   float(nodata), float(cellsize))
    else:
        if a.ndim != 2 or a.strides[1] != a.itemsize:
            raise ValueError("raster arrays must be 2-D with unit column stride")
        r = Raster(a.ctypes.data, _NP_DTYPES[a.dtype], HOST, a.shape[0], a.shape[1], a.strides[0],
                   float(nodata), float(cellsize))
    r._owner = a  # the buffer lives at least as long as its descriptor
    return r


def _stream_ptr(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream  # torch.cuda.Stream


class Context:
    """A pargo_ctx on one CUDA device (scratch, staging, counters)."""

    def __init__(self, device=0):
        self._p = ctypes.c_void_p()
        rc = lib().pargo_create(device, ctypes.byref(self._p))
        if rc:
            raise PargoError(rc, "pargo_create(%d) failed" % device)
        self.device = device
        self.moore = nbr_parse(MOORE)

    def close(self):
        if self._p:
            lib().pargo_destroy(self._p)
            self._p = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc:
            raise PargoError(rc, lib().pargo_last_error(self._p).decode(errors="replace"))

    def _nbr(self, nbr):
        return ctypes.byref(nbr if nbr is not None else self.moore)

    @property
    def last_d8_fallbacks(self):
        return lib().pargo_last_d8_fallbacks(self._p)

    def slope_d8(self, dem, slope=None, d8=None, method=SLOPE_FD, units=RATIO, dir_type=8, nbr=None, stream=None):
        """Fused slope + D8; dem/slope/d8 are Raster descriptors (see raster())."""
        self._check(lib().pargo_slope_d8(self._p, ctypes.byref(dem), ctypes.byref(slope) if slope else None,
                                         ctypes.byref(d8) if d8 else None, self._nbr(nbr), method, units, dir_type,
                                         _stream_ptr(stream)))

    def tune_focal(self, dem, reps=5):
        """Autotune the fused slope+D8 kernel on a device DEM; returns (best, ms per variant)."""
        best = ctypes.c_int(0)
        n = lib().pargo_focal_num_variants()
        times = (ctypes.c_float * n)()
        self._check(lib().pargo_tune_focal(self._p, ctypes.byref(dem), reps, ctypes.byref(best), times, n))
        return best.value, [round(t, 4) for t in times]

    def focal_variant(self, cells):
        """The kernel variant this context runs for a fused slope + D8 of `cells` cells."""
        return lib().pargo_focal_variant(self._p, cells)

    def slope(self, dem, slope, method=SLOPE_FD, units=RATIO, nbr=None, stream=None):
        self._check(lib().pargo_slope(self._p, ctypes.byref(dem), ctypes.byref(slope), self._nbr(nbr), method, units,
                                      _stream_ptr(stream)))

    def d8(self, dem, d8, dir_type=8, nbr=None, stream=None):
        self._check(lib().pargo_d8(self._p, ctypes.byref(dem), ctypes.byref(d8), self._nbr(nbr), dir_type,
                                   _stream_ptr(stream)))

    def fill(self, dem, wdem, gap=0.0005, init_level=10000.0, max_rounds=0, nbr=None, stream=None):
        opts = FillOpts(gap, init_level, max_rounds)
        stats = FillStats()
        self._check(lib().pargo_fill(self._p, ctypes.byref(dem), ctypes.byref(wdem), self._nbr(nbr),
                                     ctypes.byref(opts), ctypes.byref(stats), _stream_ptr(stream)))
        return stats

    def hydro_pipeline(self, dem, wdem=None, slope=None, d8=None, sca=None, gap=0.0005, init_level=10000.0,
                       max_rounds=0, method=SLOPE_FD, units=RATIO, contract=SCA_CONVERGED, nbr=None, stream=None):
        """Pit removal -> slope + D8 on the float64 levels -> SCA, device-resident."""
        opts = FillOpts(gap, init_level, max_rounds)
        stats = FillStats()
        ref = lambda r: ctypes.byref(r) if r is not None else None
        self._check(lib().pargo_hydro_pipeline(self._p, ctypes.byref(dem), ref(wdem), ref(slope), ref(d8), ref(sca),
                                               self._nbr(nbr), ctypes.byref(opts), method, units, contract,
                                               ctypes.byref(stats), _stream_ptr(stream)))
        return stats

    def sca(self, d8, sca, contract=SCA_CONVERGED, nbr=None, stream=None):
        self._check(lib().pargo_sca(self._p, ctypes.byref(d8), ctypes.byref(sca), self._nbr(nbr), contract,
                                    _stream_ptr(stream)))

    def twi(self, slope, sca, twi, nbr=None, stream=None):
        """Topographic wetness index ln(sca / max(slope, 1e-7)) (TWIOperator)."""
        self._check(lib().pargo_twi(self._p, ctypes.byref(slope), ctypes.byref(sca), ctypes.byref(twi),
                                    self._nbr(nbr), _stream_ptr(stream)))

    def mfd(self, dem, weights, slp_exp=1.1, nbr=None, stream=None):
        """MFD-md flow partition weights (MFDOperator) into 8 rasters."""
        if len(weights) != 8:
            raise ValueError("mfd: 8 weight rasters")
        W = (Raster * 8)(*weights)
        self._check(lib().pargo_mfd(self._p, ctypes.byref(dem), W, self._nbr(nbr), float(slp_exp),
                                    _stream_ptr(stream)))

    def sca_mfd(self, weights, sca, nbr=None, stream=None):
        """MFD specific catchment area from 8 weight rasters (scamfdmd SCAOperator)."""
        if len(weights) != 8:
            raise ValueError("sca_mfd: 8 weight rasters")
        W = (Raster * 8)(*weights)
        self._check(lib().pargo_sca_mfd(self._p, W, ctypes.byref(sca), self._nbr(nbr), _stream_ptr(stream)))

    def compute_load(self, data, load, grain, nodata_load=0.0, valid_load=1.0, compute_ring=False, nbr=None,
                     stream=None):
        """Intensity-ratio compute layer (ComputeLayer + Transformation) of one
        or several data rasters into `load`."""
        data = list(data) if isinstance(data, (list, tuple)) else [data]
        D = (Raster * len(data))(*data)
        self._check(lib().pargo_compute_load(self._p, len(data), D, self._nbr(nbr), int(grain), int(bool(compute_ring)),
                                             float(nodata_load), float(valid_load), ctypes.byref(load),
                                             _stream_ptr(stream)))

    def load_decompose(self, load, data_shape, nparts, compute_ring=False, nbr=None, stream=None):
        """Row decomposition by load: (compute rows (nparts, 2), data rectangles (nparts, 4))."""
        import numpy as np
        comp = np.zeros((nparts, 2), np.int64)
        bounds = np.zeros((nparts, 4), np.int64)
        P = ctypes.POINTER(ctypes.c_int64)
        self._check(lib().pargo_load_decompose(self._p, ctypes.byref(load), int(bool(compute_ring)),
                                               int(data_shape[0]), int(data_shape[1]), self._nbr(nbr), int(nparts),
                                               comp.ctypes.data_as(P), bounds.ctypes.data_as(P), _stream_ptr(stream)))
        return comp, bounds

    def batch_slope_d8(self, dems, slopes=None, d8s=None, method=SLOPE_FD, units=RATIO, dir_type=8, nbr=None,
                       stream=None, nodata_load=None, valid_load=None, order=None):
        """Batched slope + D8; the queue options default to the library's
        (by intensity, nodata_load 0, valid_load 1)."""
        n = len(dems)
        D = (Raster * n)(*dems)
        S = (Raster * n)(*slopes) if slopes else None
        C = (Raster * n)(*d8s) if d8s else None
        if nodata_load is None and valid_load is None and order is None:
            self._check(lib().pargo_batch_slope_d8(self._p, n, D, S, C, self._nbr(nbr), method, units, dir_type,
                                                   _stream_ptr(stream)))
            return
        o = BatchOpts(0.0 if nodata_load is None else nodata_load, 1.0 if valid_load is None else valid_load,
                      BATCH_BY_INTENSITY if order is None else order, 0)
        self._check(lib().pargo_batch_slope_d8_ex(self._p, n, D, S, C, self._nbr(nbr), method, units, dir_type,
                                                  ctypes.byref(o), _stream_ptr(stream)))

    def batch_queue(self, dems, nodata_load=0.0, valid_load=1.0, order=BATCH_BY_INTENSITY, stream=None):
        """The batched strip walk's work queue: (raster index, segment, load) arrays in queue order."""
        n = len(dems)
        D = (Raster * n)(*dems)
        o = BatchOpts(nodata_load, valid_load, order, 0)
        total = ctypes.c_int64(0)
        self._check(lib().pargo_batch_queue(self._p, n, D, ctypes.byref(o), 0, ctypes.byref(total), None, None, None,
                                            _stream_ptr(stream)))
        m = total.value
        ras = np.zeros(m, np.int32)
        seg = np.zeros(m, np.int64)
        ld = np.zeros(m, np.float64)
        self._check(lib().pargo_batch_queue(
            self._p, n, D, ctypes.byref(o), m, ctypes.byref(total), ras.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
            seg.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), ld.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
            _stream_ptr(stream)))
        return ras, seg, ld

    def batch_fill(self, dems, wdems, gap=0.0005, init_level=10000.0, max_rounds=0, nbr=None, stream=None):
        """Pit removal of many device rasters in one persistent relaxation; returns the batch's FillStats."""
        n = len(dems)
        D = (Raster * n)(*dems)
        W = (Raster * n)(*wdems)
        opts = FillOpts(gap, init_level, max_rounds)
        stats = FillStats()
        self._check(lib().pargo_batch_fill(self._p, n, D, W, self._nbr(nbr), ctypes.byref(opts), ctypes.byref(stats),
                                           _stream_ptr(stream)))
        return stats

    def slope_fwd(self, z, slope, nbr=None, stream=None):
        self._check(lib().pargo_slope_fwd(self._p, ctypes.byref(z), ctypes.byref(slope), self._nbr(nbr),
                                          _stream_ptr(stream)))

    def slope_bwd(self, z, gslope, gz, nbr=None, stream=None):
        self._check(lib().pargo_slope_bwd(self._p, ctypes.byref(z), ctypes.byref(gslope), ctypes.byref(gz),
                                          self._nbr(nbr), _stream_ptr(stream)))

    def slope_loss_grad(self, z, zref, gz, want_loss=True, nbr=None, stream=None):
        loss = ctypes.c_double(0.0)
        self._check(lib().pargo_slope_loss_grad(self._p, ctypes.byref(z), ctypes.byref(zref), ctypes.byref(gz),
                                                ctypes.byref(loss) if want_loss else None, self._nbr(nbr),
                                                _stream_ptr(stream)))
        return loss.value if want_loss else None
