"""ctypes binding of the reference library's own build (oracle/_ref, compiled
from the reference headers by oracle/build_ref.sh through ref_driver.cpp).

TEST INFRASTRUCTURE AND CPU BASELINE ONLY: imported by tests/ and by the CPU
legs of bench.py (the reference arm and the cpu_baseline sample), which time
the reference's own code on the host cores. The CUDA product never imports
this module.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LAYOUTS = ("cell", "plain")  # INTP_CELL_LAYOUT builds, and the plain layout

P = C.c_void_p
_libs = {}


def lib_path(layout):
    return os.path.join(HERE, "_ref", "libintp_ref_%s.so" % layout)


def available(layout="cell"):
    return os.path.exists(lib_path(layout))


def lib(layout="cell"):
    if layout not in _libs:
        L = C.CDLL(lib_path(layout))
        L.ref_create.restype = P
        L.ref_create.argtypes = [C.c_int, C.c_int, P, P, P, P, P, P]
        L.ref_free.argtypes = [P]
        L.ref_last_error.restype = C.c_char_p
        L.ref_eval_user.argtypes = [P, P, C.c_int64, P, C.c_int, P, C.c_int]
        L.ref_last_build_seconds.restype = C.c_double
        L.ref_locate.argtypes = [P, P, C.c_int64, P, P]
        _libs[layout] = L
    return _libs[layout]


def _p(a):
    return None if a is None else a.ctypes.data_as(P)


class RefFunction:
    """intp::InterpolationFunction<double, D, O> of the reference, built from a
    row-major value mesh on uniform axes. `build_seconds` is the time of the
    reference constructor alone (knots, factors, control-point solve on the
    reference's thread pool, and the cell layout in the cell build)."""

    def __init__(self, order, periodic, values, lo, hi, layout="cell"):
        L = lib(layout)
        v = np.ascontiguousarray(values, np.float64)
        self.dim = v.ndim
        per = np.ascontiguousarray([int(bool(p)) for p in periodic], np.int32)
        sizes = np.ascontiguousarray(v.shape, np.int64)
        lo_ = np.ascontiguousarray(lo, np.float64)
        hi_ = np.ascontiguousarray(hi, np.float64)
        self._L = L
        self.h = L.ref_create(self.dim, int(order), _p(per), _p(sizes), _p(lo_), _p(hi_), None, _p(v))
        if not self.h:
            raise RuntimeError(L.ref_last_error().decode())
        self.build_seconds = float(L.ref_last_build_seconds())

    def __del__(self):
        if getattr(self, "h", None):
            self._L.ref_free(self.h)
            self.h = None

    def outputs(self, points, derivs, nthreads=1, out=None):
        """N x K outputs: operator() for all-zero derivative rows,
        derivative() otherwise, the points split over `nthreads` threads."""
        x = np.ascontiguousarray(points, np.float64).reshape(-1, self.dim)
        k = np.ascontiguousarray(derivs, np.int32).reshape(-1, self.dim)
        if out is None:
            out = np.empty((x.shape[0], k.shape[0]), np.float64)
        self._L.ref_eval_user(self.h, _p(x), x.shape[0], _p(k), k.shape[0], _p(out), int(nthreads))
        return out

    def locate(self, points):
        x = np.ascontiguousarray(points, np.float64).reshape(-1, self.dim)
        cells = np.empty(x.shape, np.int64)
        wrapped = np.empty(x.shape, np.float64)
        self._L.ref_locate(self.h, _p(x), x.shape[0], _p(cells), _p(wrapped))
        return cells, wrapped
