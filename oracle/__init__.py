"""ctypes bindings to the test oracle (test infrastructure only).

``Oracle`` wraps the C restatement in ``oracle/pargo_oracle.c``; ``Reference``
wraps the unmodified reference operators compiled into ``oracle/_ref/``.
Only the tests, ``__graft_entry__.smoke()`` and the bench's CPU arms use this
module; the product never imports it.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_c_f32p = ctypes.POINTER(ctypes.c_float)
_c_f64p = ctypes.POINTER(ctypes.c_double)


def _p(a, t):
    return a.ctypes.data_as(t)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


MOORE_NBR = "9\n0 0 1.0\n-1 -1 1.0\n-1 0 1.0\n-1 1 1.0\n0 -1 1.0\n0 1 1.0\n1 -1 1.0\n1 0 1.0\n1 1 1.0\n"

REF_GAP = 0.0005       # apps/hydrology/pitremove/pitRemoveOperator.cpp:36
REF_INIT_LEVEL = 10000.0  # pitRemoveOperator.cpp:41


class OracleError(RuntimeError):
    pass


class Oracle:
    """The C restatement (all double precision, reference order of operations)."""

    def __init__(self, path=None):
        path = path or _build.ORACLE_SO
        if not os.path.exists(path):
            _build.build()
        lib = ctypes.CDLL(path)
        i, d, f, vp = ctypes.c_int, ctypes.c_double, ctypes.c_float, ctypes.c_void_p
        lib.orc_slope.argtypes = [vp, i, i, i, d, f, i, i, _c_f64p]
        lib.orc_d8.argtypes = [vp, i, i, i, d, i, i, _c_f64p]
        lib.orc_fill_gs.argtypes = [_c_f32p, i, i, d, d, d, i, _c_f64p, ctypes.POINTER(ctypes.c_int)]
        lib.orc_fill_pf.argtypes = [_c_f32p, i, i, d, d, d, _c_f64p]
        lib.orc_sca_sweeps.argtypes = [_c_f64p, i, i, d, i, _c_f64p, ctypes.POINTER(ctypes.c_int)]
        lib.orc_sca_topo.argtypes = [_c_f64p, i, i, d, _c_f64p, _c_f64p]
        lib.orc_twi.argtypes = [_c_f64p, _c_f64p, i, i, d, d, _c_f64p]
        lib.orc_mfd.argtypes = [vp, i, i, i, d, f, d, _c_f64p]
        lib.orc_sca_mfd.argtypes = [_c_f64p, i, i, d, _c_f64p]
        ip = ctypes.POINTER(ctypes.c_int)
        lib.orc_compute_load.argtypes = [vp, i, i, i, i, d, i, d, d, i, _c_f64p]
        lib.orc_load_decompose.argtypes = [_c_f64p, i, i, d, i, i, i, i, ip, ip]
        self.lib = lib

    @staticmethod
    def _surface(dem):
        if dem.dtype == np.float64:
            return _c(dem, np.float64), 1
        return _c(dem, np.float32), 0

    def slope(self, dem, nodata, cellsize, method=0, threads=0):
        a, f64 = self._surface(dem)
        out = np.empty(a.shape, np.float64)
        rc = self.lib.orc_slope(a.ctypes.data, f64, a.shape[0], a.shape[1], nodata, np.float32(cellsize),
                                method, threads, _p(out, _c_f64p))
        if rc:
            raise OracleError("orc_slope rc=%d" % rc)
        return out

    def d8(self, dem, nodata, dir_type=8, threads=0):
        a, f64 = self._surface(dem)
        out = np.empty(a.shape, np.float64)
        rc = self.lib.orc_d8(a.ctypes.data, f64, a.shape[0], a.shape[1], nodata, dir_type, threads, _p(out, _c_f64p))
        if rc:
            raise OracleError("orc_d8 rc=%d" % rc)
        return out

    def fill_gs(self, dem, nodata, gap=REF_GAP, init_level=REF_INIT_LEVEL, max_sweeps=1 << 30):
        a = _c(dem, np.float32)
        out = np.empty(a.shape, np.float64)
        sw = ctypes.c_int(0)
        rc = self.lib.orc_fill_gs(_p(a, _c_f32p), a.shape[0], a.shape[1], nodata, gap, init_level, max_sweeps,
                                  _p(out, _c_f64p), ctypes.byref(sw))
        if rc:
            raise OracleError("orc_fill_gs rc=%d" % rc)
        return out, sw.value

    def fill(self, dem, nodata, gap=REF_GAP, init_level=REF_INIT_LEVEL):
        a = _c(dem, np.float32)
        out = np.empty(a.shape, np.float64)
        rc = self.lib.orc_fill_pf(_p(a, _c_f32p), a.shape[0], a.shape[1], nodata, gap, init_level, _p(out, _c_f64p))
        if rc:
            raise OracleError("orc_fill_pf rc=%d" % rc)
        return out

    def sca_sweeps(self, d8, nodata, max_accum_sweeps=1):
        a = _c(d8, np.float64)
        out = np.empty(a.shape, np.float64)
        sw = ctypes.c_int(0)
        rc = self.lib.orc_sca_sweeps(_p(a, _c_f64p), a.shape[0], a.shape[1], nodata, max_accum_sweeps,
                                     _p(out, _c_f64p), ctypes.byref(sw))
        if rc:
            raise OracleError("orc_sca_sweeps rc=%d" % rc)
        return out, sw.value

    def sca(self, d8, nodata, shipped=False, allow_stall=False):
        """Converged SCA (shipped=False) or the shipped single-sweep result
        (shipped=True), by topological accumulation."""
        a = _c(d8, np.float64)
        conv = np.empty(a.shape, np.float64)
        ship = np.empty(a.shape, np.float64)
        rc = self.lib.orc_sca_topo(_p(a, _c_f64p), a.shape[0], a.shape[1], nodata, _p(conv, _c_f64p),
                                   _p(ship, _c_f64p))
        if rc and not (rc == 4 and allow_stall):
            raise OracleError("orc_sca_topo rc=%d" % rc)
        return ship if shipped else conv

    def sca_both(self, d8, nodata):
        """(converged, shipped) SCA from one topological accumulation."""
        a = _c(d8, np.float64)
        conv = np.empty(a.shape, np.float64)
        ship = np.empty(a.shape, np.float64)
        rc = self.lib.orc_sca_topo(_p(a, _c_f64p), a.shape[0], a.shape[1], nodata, _p(conv, _c_f64p),
                                   _p(ship, _c_f64p))
        if rc:
            raise OracleError("orc_sca_topo rc=%d" % rc)
        return conv, ship



    def mfd(self, dem, nodata, cellsize, slp_exp):
        """MFD-md weights (MFDOperator) as an (8, rows, cols) array: layer i is
        window position i (i < 4) or i + 1 (i >= 4)."""
        a, f64 = self._surface(dem)
        out = np.empty((8,) + a.shape, np.float64)
        rc = self.lib.orc_mfd(a.ctypes.data, f64, a.shape[0], a.shape[1], nodata, float(np.float32(cellsize)),
                              float(slp_exp), _p(out, _c_f64p))
        if rc:
            raise OracleError("orc_mfd rc=%d" % rc)
        return out

    def sca_mfd(self, weights, nodata):
        """MFD SCA as the reference's single accumulation sweep leaves it."""
        w = _c(weights, np.float64)
        out = np.empty(w.shape[1:], np.float64)
        rc = self.lib.orc_sca_mfd(_p(w, _c_f64p), w.shape[1], w.shape[2], nodata, _p(out, _c_f64p))
        if rc:
            raise OracleError("orc_sca_mfd rc=%d" % rc)
        return out

    def compute_load(self, data, nodata, grain, nodata_load, valid_load, compute_ring=False):
        """Intensity-ratio compute layer (ComputeLayer + Transformation) of one
        raster (rows, cols) or several stacked (layers, rows, cols)."""
        a = data if data.ndim == 3 else data[None]
        f64 = a.dtype == np.float64
        a = _c(a, np.float64 if f64 else np.float32)
        L, R, C = a.shape
        crows, ccols = (R - 2 + grain - 1) // grain, (C - 2 + grain - 1) // grain
        out = np.empty((crows, ccols), np.float64)
        rc = self.lib.orc_compute_load(a.ctypes.data, int(f64), L, R, C, nodata, grain, float(nodata_load),
                                       float(valid_load), int(compute_ring), _p(out, _c_f64p))
        if rc:
            raise OracleError("orc_compute_load rc=%d" % rc)
        return out

    def load_decompose(self, load, nodata, data_shape, nparts, compute_ring=False):
        """Row decomposition of a compute layer (valRowDcmp + getCompuLoad's
        mapping): (compute row ranges (nparts, 2), data rectangles (nparts, 4))."""
        a = _c(load, np.float64)
        comp = np.zeros((nparts, 2), np.int32)
        bounds = np.zeros((nparts, 4), np.int32)
        ip = ctypes.POINTER(ctypes.c_int)
        rc = self.lib.orc_load_decompose(_p(a, _c_f64p), a.shape[0], a.shape[1], nodata, int(compute_ring),
                                         data_shape[0], data_shape[1], nparts, comp.ctypes.data_as(ip),
                                         bounds.ctypes.data_as(ip))
        if rc:
            raise OracleError("orc_load_decompose rc=%d" % rc)
        return comp, bounds

    def twi(self, slope, sca, nodata, out_nodata=None):
        """Topographic wetness index ln(sca / max(slope, 1e-7)) with the
        reference's nodata rule (TWIOperator.cpp:42-69), in FP64."""
        s1 = _c(slope, np.float64)
        s2 = _c(sca, np.float64)
        out = np.empty(s1.shape, np.float64)
        rc = self.lib.orc_twi(_p(s1, _c_f64p), _p(s2, _c_f64p), s1.shape[0], s1.shape[1], nodata,
                              nodata if out_nodata is None else out_nodata, _p(out, _c_f64p))
        if rc:
            raise OracleError("orc_twi rc=%d" % rc)
        return out
class Reference:
    """The unmodified reference operators (available where the reference tree is)."""

    def __init__(self, path=None):
        path = path or _build.REF_SO
        if not os.path.exists(path):
            if not _build.reference_available():
                raise OracleError("reference build unavailable: reference tree absent")
            _build.build()
        lib = ctypes.CDLL(path)
        i, d, vp, cp = ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_char_p
        lib.ref_slope.argtypes = [cp, _c_f32p, i, i, d, d, i, i, _c_f64p]
        lib.ref_d8.argtypes = [cp, vp, i, i, i, d, d, i, i, _c_f64p]
        lib.ref_fill.argtypes = [cp, _c_f32p, i, i, d, d, _c_f64p, ctypes.POINTER(ctypes.c_int)]
        lib.ref_sca.argtypes = [cp, _c_f64p, i, i, d, d, i, _c_f64p, ctypes.POINTER(ctypes.c_int)]
        lib.ref_twi.argtypes = [cp, _c_f64p, _c_f64p, i, i, d, d, _c_f64p]
        ip = ctypes.POINTER(ctypes.c_int)
        lib.ref_compute_load.argtypes = [cp, _c_f32p, i, i, d, d, i, d, d, i, i, _c_f64p, ip, ip, ip, ip]
        self.lib = lib
        self.mfd_lib = None
        if os.path.exists(_build.REF_MFD_SO):
            m = ctypes.CDLL(_build.REF_MFD_SO)
            m.ref_mfd.argtypes = [cp, _c_f32p, i, i, d, d, d, _c_f64p]
            m.ref_sca_mfd.argtypes = [cp, _c_f64p, i, i, d, d, _c_f64p]
            self.mfd_lib = m
        self._nbr = os.path.join(_build.REF_OUT, "moore.nbr")
        with open(self._nbr, "w") as fh:
            fh.write(MOORE_NBR)

    @staticmethod
    def available():
        return os.path.exists(_build.REF_SO) or _build.reference_available()

    def slope(self, dem, nodata, cellsize, method=0, threads=0):
        a = _c(dem, np.float32)
        out = np.empty(a.shape, np.float64)
        rc = self.lib.ref_slope(self._nbr.encode(), _p(a, _c_f32p), a.shape[0], a.shape[1], nodata, cellsize,
                                method, threads, _p(out, _c_f64p))
        if rc:
            raise OracleError("ref_slope rc=%d" % rc)
        return out

    def d8(self, dem, nodata, cellsize=1.0, dir_type=8, threads=0):
        f64 = 1 if dem.dtype == np.float64 else 0
        a = _c(dem, np.float64 if f64 else np.float32)
        out = np.empty(a.shape, np.float64)
        rc = self.lib.ref_d8(self._nbr.encode(), a.ctypes.data, f64, a.shape[0], a.shape[1], nodata, cellsize,
                             dir_type, threads, _p(out, _c_f64p))
        if rc:
            raise OracleError("ref_d8 rc=%d" % rc)
        return out

    def fill(self, dem, nodata, cellsize=1.0):
        a = _c(dem, np.float32)
        out = np.empty(a.shape, np.float64)
        sw = ctypes.c_int(0)
        rc = self.lib.ref_fill(self._nbr.encode(), _p(a, _c_f32p), a.shape[0], a.shape[1], nodata, cellsize,
                               _p(out, _c_f64p), ctypes.byref(sw))
        if rc:
            raise OracleError("ref_fill rc=%d" % rc)
        return out, sw.value

    def sca(self, d8, nodata, cellsize=1.0, converged=True):
        a = _c(d8, np.float64)
        out = np.empty(a.shape, np.float64)
        sw = ctypes.c_int(0)
        rc = self.lib.ref_sca(self._nbr.encode(), _p(a, _c_f64p), a.shape[0], a.shape[1], nodata, cellsize,
                              1 if converged else 0, _p(out, _c_f64p), ctypes.byref(sw))
        if rc:
            raise OracleError("ref_sca rc=%d" % rc)
        return out, sw.value

    def mfd(self, dem, nodata, cellsize, slp_exp):
        a = _c(dem, np.float32)
        out = np.empty((8,) + a.shape, np.float64)
        rc = self.mfd_lib.ref_mfd(self._nbr.encode(), _p(a, _c_f32p), a.shape[0], a.shape[1], nodata, cellsize,
                                  float(slp_exp), _p(out, _c_f64p))
        if rc:
            raise OracleError("ref_mfd rc=%d" % rc)
        return out

    def sca_mfd(self, weights, nodata, cellsize=1.0):
        w = _c(weights, np.float64)
        out = np.empty(w.shape[1:], np.float64)
        rc = self.mfd_lib.ref_sca_mfd(self._nbr.encode(), _p(w, _c_f64p), w.shape[1], w.shape[2], nodata, cellsize,
                                      _p(out, _c_f64p))
        if rc:
            raise OracleError("ref_sca_mfd rc=%d" % rc)
        return out

    def twi(self, slope, sca, nodata, cellsize=1.0):
        s1 = _c(slope, np.float64)
        s2 = _c(sca, np.float64)
        out = np.empty(s1.shape, np.float64)
        rc = self.lib.ref_twi(self._nbr.encode(), _p(s1, _c_f64p), _p(s2, _c_f64p), s1.shape[0], s1.shape[1], nodata,
                              cellsize, _p(out, _c_f64p))
        if rc:
            raise OracleError("ref_twi rc=%d" % rc)
        return out

    def compute_load(self, data, nodata, grain, nodata_load, valid_load, compute_ring=False, nparts=0,
                     cellsize=1.0):
        """(compute layer, compute row ranges (nparts, 2), rank 0's data rectangle)
        from the reference ComputeLayer / Transformation / DeComposition."""
        a = _c(data, np.float32)
        R, C = a.shape
        crows, ccols = (R - 2 + grain - 1) // grain, (C - 2 + grain - 1) // grain
        out = np.empty((crows, ccols), np.float64)
        comp = np.zeros((max(nparts, 1), 2), np.int32)
        rank0 = np.zeros(4, np.int32)
        cr, cc = ctypes.c_int(), ctypes.c_int()
        ip = ctypes.POINTER(ctypes.c_int)
        rc = self.lib.ref_compute_load(self._nbr.encode(), _p(a, _c_f32p), R, C, nodata, cellsize, grain,
                                       float(nodata_load), float(valid_load), int(compute_ring), nparts,
                                       _p(out, _c_f64p), ctypes.byref(cr), ctypes.byref(cc), comp.ctypes.data_as(ip),
                                       rank0.ctypes.data_as(ip))
        if rc:
            raise OracleError("ref_compute_load rc=%d" % rc)
        assert (cr.value, cc.value) == out.shape
        return out, comp[:nparts], rank0
