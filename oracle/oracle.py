"""ctypes binding of the C oracle (intp_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() and by
the CPU-baseline leg of bench.py, as the checker / the timed CPU restatement of
the reference algorithm. The CUDA product never imports this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libintp_oracle.so")

P = C.c_void_p


def build(force=False):
    """Compile the oracle for the host it runs on (gcc, no FMA contraction)."""
    src = os.path.join(HERE, "intp_oracle.c")
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(src):
        return LIB_PATH
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-std=c11", "-O3", "-fPIC", "-shared", "-ffp-contract=off",
                           "-pthread", src, "-o", tmp, "-lm"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.or_create.restype = P
        L.or_create.argtypes = [C.c_int, C.c_int, P, P, P, P, P]
        L.or_create_from_knots.restype = P
        L.or_create_from_knots.argtypes = [C.c_int, C.c_int, P, P, P, P, P]
        L.or_free.argtypes = [P]
        L.or_last_error.restype = C.c_char_p
        L.or_interpolate.argtypes = [P, P, C.c_int]
        L.or_set_control_points.argtypes = [P, P]
        L.or_get_control_points.argtypes = [P, P]
        L.or_num_knots.restype = C.c_int64
        L.or_num_knots.argtypes = [P, C.c_int]
        L.or_get_knots.argtypes = [P, C.c_int, P]
        L.or_get_range.argtypes = [P, C.c_int, P, P]
        L.or_get_dx.restype = C.c_double
        L.or_get_dx.argtypes = [P, C.c_int]
        L.or_eval.argtypes = [P, P, C.c_int64, P, C.c_int]
        L.or_eval_deriv.argtypes = [P, P, C.c_int64, P, C.c_int, P, C.c_int]
        L.or_locate.argtypes = [P, P, C.c_int64, P, P]
        L.or_in_range.argtypes = [P, P]
        L.or_band_solve_dense.argtypes = [C.c_int64, C.c_int, C.c_int, C.c_int, P, P]
        L.or_base_spline_value.argtypes = [P, C.c_int64, C.c_double, C.c_int, C.c_int, P]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(P)


class Spline:
    """Oracle spline: knots, factors and control points of one table."""

    def __init__(self, dim, order, periodic, sizes, lo=None, hi=None, coords=None):
        L = lib()
        self.dim, self.order = dim, order
        per = np.ascontiguousarray([int(bool(v)) for v in periodic], np.int32)
        sz = np.ascontiguousarray(sizes, np.int64)
        lo_ = np.ascontiguousarray(lo if lo is not None else [0.0] * dim, np.float64)
        hi_ = np.ascontiguousarray(hi if hi is not None else [0.0] * dim, np.float64)
        self._coords = [None if c is None else np.ascontiguousarray(c, np.float64)
                        for c in (coords or [None] * dim)]
        cptr = (P * dim)(*[None if c is None else c.ctypes.data for c in self._coords])
        self.h = L.or_create(dim, order, _p(per), _p(sz), _p(lo_), _p(hi_), cptr)
        if not self.h:
            raise ValueError(L.or_last_error().decode())
        self.sizes = [int(s) for s in sizes]

    @classmethod
    def from_knots(cls, dim, order, periodic, ncp, knots, ctrl):
        self = cls.__new__(cls)
        L = lib()
        self.dim, self.order = dim, order
        per = np.ascontiguousarray([int(bool(v)) for v in periodic], np.int32)
        n = np.ascontiguousarray(ncp, np.int64)
        self._knots = [np.ascontiguousarray(k, np.float64) for k in knots]
        nk = np.ascontiguousarray([len(k) for k in knots], np.int64)
        kp = (P * dim)(*[k.ctypes.data for k in self._knots])
        c = np.ascontiguousarray(ctrl, np.float64)
        self.h = L.or_create_from_knots(dim, order, _p(per), _p(n), kp, _p(nk), _p(c))
        self.sizes = [int(s) for s in ncp]
        return self

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_free(self.h)
            self.h = None

    def interpolate(self, values, nthreads=1):
        v = np.ascontiguousarray(values, np.float64).ravel()
        assert v.size == int(np.prod(self.sizes))
        if lib().or_interpolate(self.h, _p(v), int(nthreads)) != 0:
            raise RuntimeError(lib().or_last_error().decode())
        return self

    def control_points(self):
        out = np.zeros(int(np.prod(self.sizes)))
        lib().or_get_control_points(self.h, _p(out))
        return out.reshape(self.sizes)

    def set_control_points(self, ctrl):
        c = np.ascontiguousarray(ctrl, np.float64).ravel()
        lib().or_set_control_points(self.h, _p(c))

    def knots(self, axis):
        out = np.zeros(lib().or_num_knots(self.h, axis))
        lib().or_get_knots(self.h, axis, _p(out))
        return out

    def range(self, axis):
        a, b = C.c_double(), C.c_double()
        lib().or_get_range(self.h, axis, C.byref(a), C.byref(b))
        return a.value, b.value

    def dx(self, axis):
        return lib().or_get_dx(self.h, axis)

    def eval(self, points, nthreads=1):
        x = np.ascontiguousarray(points, np.float64).reshape(-1, self.dim)
        out = np.zeros(x.shape[0])
        lib().or_eval(self.h, _p(x), x.shape[0], _p(out), int(nthreads))
        return out

    def derivative(self, points, derivs, nthreads=1):
        x = np.ascontiguousarray(points, np.float64).reshape(-1, self.dim)
        k = np.ascontiguousarray(derivs, np.int32).reshape(-1, self.dim)
        out = np.zeros((x.shape[0], k.shape[0]))
        lib().or_eval_deriv(self.h, _p(x), x.shape[0], _p(k), k.shape[0], _p(out), int(nthreads))
        return out

    def locate(self, points):
        x = np.ascontiguousarray(points, np.float64).reshape(-1, self.dim)
        cells = np.zeros(x.shape, np.int64)
        wrapped = np.zeros(x.shape)
        lib().or_locate(self.h, _p(x), x.shape[0], _p(cells), _p(wrapped))
        return cells, wrapped

    def in_range(self, point):
        x = np.ascontiguousarray(point, np.float64)
        return bool(lib().or_in_range(self.h, _p(x)))


def band_solve_dense(a, b, p, q, cyclic):
    a = np.ascontiguousarray(a, np.float64)
    x = np.ascontiguousarray(b, np.float64).copy()
    if lib().or_band_solve_dense(a.shape[0], p, q, int(cyclic), _p(a), _p(x)) != 0:
        raise ValueError(lib().or_last_error().decode())
    return x


def base_spline_value(knots, seg, x, order, spline_order=None):
    k = np.ascontiguousarray(knots, np.float64)
    out = np.zeros(order + 1)
    lib().or_base_spline_value(_p(k), seg, x, order,
                               order if spline_order is None else spline_order, _p(out))
    return out
