"""GB300-native B-spline interpolation (hot path of 12ff54e/BSplineInterpolation).

Python host mirror of the reference's C++ interface (src/include/
Interpolation.hpp, InterpolationTemplate.hpp, BandLU.hpp) over the CUDA
library's C-ABI (include/intp_gpu.h). The same interface exists as a
header-only C++ drop-in under include/intp/.

    f = InterpolationFunction(3, [False, False], mesh, (0.0, 1.0), (0.0, 2.0))
    f(0.3, 1.1)                      # operator()
    f.derivative_at((0.3, 1.1), 1, 0)  # range-checked derivative
    f.evaluate(points, derivs=[[0, 0], [1, 0]])  # batched, device or host

There is no CPU fallback: the CUDA library must be built (build.build()).
"""
import ctypes as C

import numpy as np

from . import _lib
from ._lib import IntpDomainError, IntpError

__all__ = [
    "InterpolationFunction",
    "InterpolationFunction1D",
    "InterpolationFunctionTemplate",
    "InterpolationFunctionTemplate1D",
    "BandLU",
    "TableBatch",
    "Server",
    "EvalProxy",
    "host_empty",
    "IntpError",
    "IntpDomainError",
]

_PRECISIONS = {"fp64": _lib.PRECISION_FP64, "mixed": _lib.PRECISION_MIXED}


def _torch():
    try:
        import torch
        return torch
    except ImportError:
        return None


def _is_cuda_tensor(x):
    t = _torch()
    return t is not None and isinstance(x, t.Tensor) and x.is_cuda


def _stream_ptr(stream):
    if stream is None:
        t = _torch()
        if t is not None and t.cuda.is_available() and t.cuda.is_initialized():
            return C.c_void_p(t.cuda.current_stream().cuda_stream)
        return None
    if isinstance(stream, int):
        return C.c_void_p(stream)
    return C.c_void_p(stream.cuda_stream)


def _is_range(r):
    return isinstance(r, (tuple, list)) and len(r) == 2 and all(np.isscalar(v) for v in r)


def _make_desc(order, periodicity, mesh_dims, x_ranges, precision, refine_steps, channels=1):
    """intp_table_desc of one table; returns (desc, arrays to keep alive, dims,
    periodicity)."""
    dims = [int(v) for v in np.atleast_1d(mesh_dims)]
    D = len(dims)
    if len(x_ranges) != D:
        raise ValueError("need one x range per dimension")
    if periodicity is None:
        periodicity = [False] * D
    periodicity = [bool(v) for v in np.atleast_1d(periodicity)]
    if len(periodicity) != D:
        raise ValueError("need one periodicity flag per dimension")
    desc = _lib.TableDesc()
    desc.dim = D
    desc.order = int(order)
    desc.precision = _PRECISIONS[precision]
    desc.refine_steps = int(refine_steps)
    desc.channels = int(channels)
    keep = []
    for d in range(D):
        desc.periodic[d] = int(periodicity[d])
        desc.size[d] = dims[d]
        r = x_ranges[d]
        if _is_range(r):
            desc.range_lo[d] = float(r[0])
            desc.range_hi[d] = float(r[1])
            desc.coords[d] = None
        else:
            c = np.ascontiguousarray(np.asarray(r, np.float64))
            if c.ndim != 1 or c.size != dims[d] + (1 if periodicity[d] else 0):
                raise ValueError("axis %d: expected %d coordinates" %
                                 (d, dims[d] + (1 if periodicity[d] else 0)))
            keep.append(c)
            desc.coords[d] = c.ctypes.data
    return desc, keep, dims, periodicity


class _HostBlock:
    """Owner of one intp_host_alloc block; freed when the last view goes."""

    def __init__(self, nbytes):
        self.ptr = C.c_void_p()
        _lib.check(_lib.load().intp_host_alloc(nbytes, C.byref(self.ptr)))

    def __del__(self):
        if self.ptr:
            _lib.load().intp_host_free(self.ptr)
            self.ptr = C.c_void_p()


def host_empty(shape, dtype=np.float64):
    """An uninitialised numpy array in page-locked host memory from
    intp_host_alloc: the host-buffer entry points (InterpolationFunction.
    evaluate on numpy points, intp_eval_host) copy it to and from the device
    at the full host link rate. The memory is released with the last view of
    the array (torch.from_numpy views keep it too)."""
    dt = np.dtype(dtype)
    n = int(np.prod(shape))
    block = _HostBlock(max(1, n) * dt.itemsize)
    buf = (C.c_char * (max(1, n) * dt.itemsize)).from_address(block.ptr.value)
    buf._intp_block = block  # the ctypes buffer owns the allocation
    return np.frombuffer(buf, dtype=dt, count=n).reshape(shape)


class InterpolationFunctionTemplate:
    """Knots and per-axis band LU factors for a mesh shape; solves for control
    points of any value mesh of that shape.

    Mirrors InterpolationFunctionTemplate (InterpolationTemplate.hpp:32-581):
    constructor (:60-79) and interpolate (:118-143). `x_ranges` holds, per
    axis, either (x_min, x_max) for a uniform axis or a 1-D array of sample
    coordinates for a non-uniform one (size + 1 entries on a periodic axis).
    """

    def __init__(self, order, periodicity, mesh_dims, *x_ranges, precision="fp64",
                 refine_steps=-1, channels=1):
        lib = _lib.load()
        desc, self._coords, dims, periodicity = _make_desc(order, periodicity, mesh_dims, x_ranges,
                                                           precision, refine_steps, channels)
        D = len(dims)
        self.channels = max(1, int(channels))
        h = C.c_void_p()
        _lib.check(lib.intp_table_create(C.byref(desc), C.byref(h)))
        self._h = h
        self.dim = D
        self.order = int(order)
        self.dims = dims
        self.precision = precision
        self._periodicity = periodicity
        self._x_ranges = x_ranges
        self._refine = int(refine_steps)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.load().intp_table_destroy(h)
            self._h = None

    def _solve(self, mesh, stream=None):
        lib = _lib.load()
        if _is_cuda_tensor(mesh):
            torch = _torch()
            m = mesh.to(torch.float64).contiguous()
            if m.numel() != int(np.prod(self.dims)) * self.channels:
                raise ValueError("mesh shape mismatch")
            _lib.check(lib.intp_table_interpolate(self._h, C.c_void_p(m.data_ptr()), 1,
                                                  _stream_ptr(stream)))
            self._keep = m
        else:
            m = np.ascontiguousarray(np.asarray(mesh, np.float64))
            if m.size != int(np.prod(self.dims)) * self.channels:
                raise ValueError("mesh shape mismatch")
            _lib.check(lib.intp_table_interpolate(self._h, m.ctypes.data, 0, _stream_ptr(stream)))
            _lib.check(lib.intp_stream_synchronize(_stream_ptr(stream)))

    def eval_proxy(self, points, stream=None):
        """Spans and basis weights of `points` (CUDA tensor, N x dim), reusable
        for every function interpolated from this template
        (InterpolationTemplate.hpp:145-176); see EvalProxy."""
        return EvalProxy(self._h, self.dim, points, stream)

    def interpolate(self, mesh, stream=None):
        """Solve for control points of `mesh` (InterpolationTemplate.hpp:118-143);
        returns a new InterpolationFunction with its own device table."""
        f = InterpolationFunction.__new__(InterpolationFunction)
        f._template = InterpolationFunctionTemplate(self.order, self._periodicity, self.dims,
                                                    *self._x_ranges, precision=self.precision,
                                                    refine_steps=self._refine, channels=self.channels)
        f._template._solve(mesh, stream)
        f._init_from_template()
        return f


class InterpolationFunction:
    """Tensor-product B-spline interpolant of a value mesh, on the GPU.

    Mirrors InterpolationFunction<T, D, O, U> (Interpolation.hpp:17-507):
    construction from (periodicity, mesh, x_ranges...) (:92-107), operator()
    (:132-146), at (:153-169), derivative (:177-205), derivative_at (:213-244),
    periodicity / uniform / range (:248-258), get_order (:267). Batched
    evaluation is `evaluate`.
    """

    def __init__(self, order, periodicity, mesh, *x_ranges, precision="fp64", refine_steps=-1,
                 stream=None, vector=False):
        """vector=True: the last axis of `mesh` holds the C components of a
        vector-valued T (the reference's InterpolationFunction<Vec<C, .>, D, O>);
        evaluations then return C values per output."""
        if _is_cuda_tensor(mesh):
            dims = list(mesh.shape)
        else:
            dims = list(np.shape(mesh))
        channels = 1
        if vector:
            channels = dims[-1]
            dims = dims[:-1]
        if len(x_ranges) == 1 and len(dims) > 1 and not _is_range(x_ranges[0]):
            x_ranges = tuple(x_ranges[0])
        self._template = InterpolationFunctionTemplate(order, periodicity, dims, *x_ranges,
                                                       precision=precision,
                                                       refine_steps=refine_steps, channels=channels)
        self._template._solve(mesh, stream)
        self._init_from_template()

    def _init_from_template(self):
        lib = _lib.load()
        t = self._template
        self.dim = t.dim
        self.order = t.order
        self.precision = t.precision
        self.channels = t.channels
        self._h = t._h
        self._range = []
        self._uniform = []
        self._per = []
        for d in range(self.dim):
            nk, lo, hi, per, uni = (C.c_int64(), C.c_double(), C.c_double(), C.c_int32(),
                                    C.c_int32())
            _lib.check(lib.intp_table_axis_info(self._h, d, C.byref(nk), C.byref(lo), C.byref(hi),
                                                C.byref(per), C.byref(uni)))
            self._range.append((lo.value, hi.value))
            self._uniform.append(bool(uni.value))
            self._per.append(bool(per.value))

    # -- properties (Interpolation.hpp:248-267) --
    def periodicity(self, d):
        return self._per[d]

    def uniform(self, d):
        return self._uniform[d]

    def range(self, d):
        return self._range[d]

    def get_order(self):
        return self.order

    def knots(self, d):
        lib = _lib.load()
        nk = C.c_int64()
        _lib.check(lib.intp_table_axis_info(self._h, d, C.byref(nk), None, None, None, None))
        out = np.zeros(nk.value)
        _lib.check(lib.intp_table_knots(self._h, d, out.ctypes.data))
        return out

    def control_points(self):
        C = self.channels
        out = np.zeros(int(np.prod(self._template.dims)) * C)
        _lib.check(_lib.load().intp_table_get_control_points(self._h, out.ctypes.data))
        return out.reshape(self._template.dims + ([C] if C > 1 else []))

    # -- batched evaluation --
    def evaluate(self, points, derivs=None, out=None, out_dtype=None, stream=None):
        """Values (derivs None) or derivatives (derivs: K x D orders) at N
        points (N x D). CUDA tensors stay on the device (result: N x K CUDA
        tensor); host arrays take the host path (result: N x K numpy array)."""
        lib = _lib.load()
        D = self.dim
        if out_dtype is None:
            out_dtype = "f32" if self.precision == "mixed" else "f64"
        od = _lib.F32 if out_dtype == "f32" else _lib.F64
        if derivs is None:
            kp, K = None, 1
            karr = None
        else:
            karr = np.ascontiguousarray(np.asarray(derivs, np.int32).reshape(-1, D))
            K = karr.shape[0]
            kp = karr.ctypes.data
        # vector-valued tables: C values per output (shape N x K x C)
        shape = (K,) if self.channels == 1 else (K, self.channels)
        if _is_cuda_tensor(points):
            torch = _torch()
            pts = points.to(torch.float64).contiguous().reshape(-1, D)
            n = pts.shape[0]
            if out is None:
                out = torch.empty((n,) + shape, dtype=torch.float32 if od == _lib.F32 else torch.float64,
                                  device=pts.device)
            _lib.check(lib.intp_eval(self._h, C.c_void_p(pts.data_ptr()), n, kp, K,
                                     C.c_void_p(out.data_ptr()), od, _stream_ptr(stream)))
            return out
        pts = np.ascontiguousarray(np.asarray(points, np.float64).reshape(-1, D))
        n = pts.shape[0]
        res = np.zeros((n,) + shape, np.float32 if od == _lib.F32 else np.float64)
        _lib.check(lib.intp_eval_host(self._h, pts.ctypes.data, n, kp, K, res.ctypes.data, od,
                                      _stream_ptr(stream)))
        return res

    def eval_proxy(self, points, stream=None):
        """Spans and basis weights of `points` for this function's knots
        (Interpolation.hpp:493-503); see EvalProxy."""
        return EvalProxy(self._h, self.dim, points, stream)

    def locate(self, points, stream=None):
        """Knot-span indices (N x D int64) and wrapped coordinates, for CUDA
        tensors of points (BSpline.hpp:125-157)."""
        torch = _torch()
        lib = _lib.load()
        pts = points.to(torch.float64).contiguous().reshape(-1, self.dim)
        cells = torch.empty(pts.shape, dtype=torch.int64, device=pts.device)
        wrapped = torch.empty(pts.shape, dtype=torch.float64, device=pts.device)
        _lib.check(lib.intp_locate(self._h, C.c_void_p(pts.data_ptr()), pts.shape[0],
                                   C.c_void_p(cells.data_ptr()), C.c_void_p(wrapped.data_ptr()),
                                   _stream_ptr(stream)))
        return cells, wrapped

    def locate_binned(self, points, stream=None):
        """Knot-span indices (N x D int64) as the binned evaluation path
        computes them (its own locate kernel, records decoded); mixed scalar
        tables of dimension 1..3 only."""
        torch = _torch()
        lib = _lib.load()
        pts = points.to(torch.float64).contiguous().reshape(-1, self.dim)
        cells = torch.empty(pts.shape, dtype=torch.int64, device=pts.device)
        _lib.check(lib.intp_locate_binned(self._h, C.c_void_p(pts.data_ptr()), pts.shape[0],
                                          C.c_void_p(cells.data_ptr()), _stream_ptr(stream)))
        return cells

    def check_range(self, points, stream=None):
        """Index of the first point outside a non-periodic axis range, or -1."""
        torch = _torch()
        lib = _lib.load()
        pts = points.to(torch.float64).contiguous().reshape(-1, self.dim)
        bad = C.c_int64()
        _lib.check(lib.intp_check_range(self._h, C.c_void_p(pts.data_ptr()), pts.shape[0],
                                        C.byref(bad), _stream_ptr(stream)))
        return bad.value

    # -- single-point API of the reference --
    def _coord(self, coords):
        if len(coords) == 1 and np.ndim(coords[0]) == 1:
            coords = tuple(coords[0])
        if len(coords) != self.dim:
            raise ValueError("expected %d coordinates" % self.dim)
        return np.asarray(coords, np.float64)

    def _boundary_check(self, c):
        for d in range(self.dim):
            lo, hi = self._range[d]
            if not self._per[d] and (c[d] < lo or c[d] > hi):
                raise IntpDomainError(_lib.ERR_DOMAIN,
                                      "Given coordinate out of interpolation function range!")

    def _one(self, v):
        return float(v) if self.channels == 1 else np.asarray(v)

    def __call__(self, *coords):
        c = self._coord(coords)
        return self._one(self.evaluate(c.reshape(1, -1), out_dtype="f64")[0, 0])

    def at(self, *coords):
        c = self._coord(coords)
        self._boundary_check(c)
        return self._one(self.evaluate(c.reshape(1, -1), out_dtype="f64")[0, 0])

    def _derivs(self, coord, orders):
        if len(orders) == 1 and np.ndim(orders[0]) == 1:
            orders = tuple(orders[0])
        if len(orders) != self.dim:
            raise ValueError("expected %d derivative orders" % self.dim)
        return np.asarray(coord, np.float64).reshape(1, -1), np.asarray(orders, np.int32)

    def derivative(self, coord, *orders):
        c, k = self._derivs(coord, orders)
        return self._one(self.evaluate(c, derivs=k.reshape(1, -1), out_dtype="f64")[0, 0])

    def derivative_at(self, coord, *orders):
        c, k = self._derivs(coord, orders)
        self._boundary_check(c[0])
        return self._one(self.evaluate(c, derivs=k.reshape(1, -1), out_dtype="f64")[0, 0])


class InterpolationFunction1D(InterpolationFunction):
    """1-D convenience form (Interpolation.hpp:509-540). Without an x range the
    samples sit at 0, 1, 2, ...: the range is (0, n-1), or (0, n) when periodic
    (INTP_PERIODIC_NO_DUMMY_POINT)."""

    def __init__(self, order, f, x_range=None, periodic=False, **kw):
        f = f if _is_cuda_tensor(f) else np.asarray(f, np.float64)
        n = f.shape[0]
        if f.ndim == 2:
            kw.setdefault("vector", True)  # n samples of a vector-valued function
        if x_range is None:
            x_range = (0.0, float(n - (0 if periodic else 1)))
        super().__init__(order, [periodic], f, x_range, **kw)


class InterpolationFunctionTemplate1D(InterpolationFunctionTemplate):
    """InterpolationTemplate.hpp:583-604: range defaults to (0, f_length - 1)."""

    def __init__(self, order, f_length, x_range=None, periodic=False, **kw):
        if x_range is None:
            x_range = (0.0, float(f_length - 1))
        super().__init__(order, [periodic], [f_length], x_range, **kw)


class EvalProxy:
    """Precomputed knot spans and value weights of N points (device memory),
    reusable across every function that shares the knots -- the reference's
    eval_proxy / pre_calc_coef (InterpolationTemplate.hpp:145-176,
    BSpline.hpp:250-296) for a whole point set. proxy(f) gives f's values at
    the points (N); proxy(f, g, ...) evaluates all of them in one launch and
    gives an N x k tensor. Scalar tables of dimension 1..3."""

    def __init__(self, table_handle, dim, points, stream=None):
        torch = _torch()
        lib = _lib.load()
        pts = points.to(torch.float64).contiguous().reshape(-1, dim)
        self.npts = pts.shape[0]
        self.dim = dim
        h = C.c_void_p()
        _lib.check(lib.intp_proxy_create(table_handle, C.c_void_p(pts.data_ptr()), self.npts,
                                         _stream_ptr(stream), C.byref(h)))
        self._h = h
        self._device = pts.device

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.load().intp_proxy_destroy(h)
            self._h = None

    def __call__(self, *functions, out_dtype=None, stream=None):
        torch = _torch()
        lib = _lib.load()
        if not functions:
            raise ValueError("at least one function")
        if out_dtype is None:
            out_dtype = "f32" if functions[0].precision == "mixed" else "f64"
        dt = torch.float32 if out_dtype == "f32" else torch.float64
        out = torch.empty((self.npts, len(functions)), dtype=dt, device=self._device)
        handles = (C.c_void_p * len(functions))(*[f._h.value for f in functions])
        _lib.check(lib.intp_proxy_eval(self._h, handles, len(functions), C.c_void_p(out.data_ptr()),
                                       _lib.F32 if out_dtype == "f32" else _lib.F64, _stream_ptr(stream)))
        return out[:, 0] if len(functions) == 1 else out


class BandLU:
    """Band LU without pivoting (BandLU.hpp), solved on the GPU.

    `band` is n x (1+p+q) in the reference's storage (A(i,j) =
    band[j, i+q-j]); cyclic matrices add `right` ((n-q-1) x p) and `bottom`
    ((n-p-1) x q) corner blocks (ExtendedBandMatrix)."""

    def __init__(self, band, p, q, right=None, bottom=None):
        lib = _lib.load()
        band = np.ascontiguousarray(band, np.float64)
        n = band.shape[0]
        cyclic = right is not None
        self._r = None if right is None else np.ascontiguousarray(right, np.float64)
        self._b = None if bottom is None else np.ascontiguousarray(bottom, np.float64)
        h = C.c_void_p()
        _lib.check(lib.intp_bandlu_create(n, p, q, int(cyclic), band.ctypes.data,
                                          None if self._r is None else self._r.ctypes.data,
                                          None if self._b is None else self._b.ctypes.data,
                                          C.byref(h)))
        self._h = h
        self.n = n

    @classmethod
    def from_dense(cls, a, p, q, cyclic=False):
        """Band storage from a dense matrix (only band / side-band entries read)."""
        a = np.asarray(a, np.float64)
        n = a.shape[0]
        band = np.zeros((n, 1 + p + q))
        for i in range(n):
            for j in range(max(0, i - p), min(n, i + q + 1)):
                band[j, i + q - j] = a[i, j]
        if not cyclic:
            return cls(band, p, q)
        right = np.zeros((max(n - q - 1, 0), p))
        bottom = np.zeros((max(n - p - 1, 0), q))
        for i in range(n):
            for j in range(n):
                if j >= max(n - p, i + q + 1):
                    right[i, j + p - n] = a[i, j]
                elif i >= max(n - q, j + p + 1):
                    bottom[j, i + q - n] = a[i, j]
        return cls(band, p, q, right, bottom)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.load().intp_bandlu_destroy(h)
            self._h = None

    def solve(self, x, stream=None):
        """Solves in place along axis 0 of a CUDA tensor (n, ...) of float64;
        for a host array returns the solution (copied through the device)."""
        lib = _lib.load()
        torch = _torch()
        if _is_cuda_tensor(x):
            assert x.dtype == torch.float64 and x.is_contiguous() and x.shape[0] == self.n
            inner = x.numel() // self.n
            _lib.check(lib.intp_bandlu_solve(self._h, C.c_void_p(x.data_ptr()), 1, inner,
                                             _stream_ptr(stream)))
            return x
        xt = torch.tensor(np.asarray(x, np.float64), device="cuda")
        self.solve(xt, stream)
        torch.cuda.synchronize()
        return xt.cpu().numpy()


class TableBatch:
    """Many independent tables built and evaluated together (intp_batch_*).

    `tables` is a sequence of (order, periodicity, mesh_dims, x_ranges)
    tuples, one per table, with the meaning of InterpolationFunctionTemplate's
    arguments (dimension 1..3), optionally with a fifth entry C > 1 for a
    vector-valued table of C components (its values hold the C components of
    each mesh point consecutively). Every table of a batch has one precision.
    The reference builds such tables one InterpolationFunction at a time
    (InterpolationTemplate.hpp:60-143); here one launch per axis pass solves
    all of them, and one launch per (dimension, order) class evaluates them.
    """

    def __init__(self, tables, precision="mixed", refine_steps=-1):
        lib = _lib.load()
        n = len(tables)
        descs = (_lib.TableDesc * n)()
        self._keep = []
        self.dims = []
        self.orders = []
        self.channels = []
        for i, t in enumerate(tables):
            order, periodicity, mesh_dims, x_ranges = t[:4]
            ch = int(t[4]) if len(t) > 4 else 1
            desc, keep, dims, _ = _make_desc(order, periodicity, mesh_dims, list(x_ranges), precision,
                                             refine_steps, ch)
            descs[i] = desc
            self._keep.extend(keep)
            self.dims.append(dims)
            self.orders.append(int(order))
            self.channels.append(max(1, ch))
        h = C.c_void_p()
        _lib.check(lib.intp_batch_create(descs, n, C.byref(h)))
        self._h = h
        self.ntables = n
        self.precision = precision
        self.sizes = [int(np.prod(d)) * c for d, c in zip(self.dims, self.channels)]
        self.offsets = np.concatenate([[0], np.cumsum(self.sizes)]).astype(np.int64)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.load().intp_batch_destroy(h)
            self._h = None

    def build(self, values, stream=None):
        """Solves every table's control points. `values`: one flat array of all
        meshes in table order (a CUDA tensor stays on the device), or a list
        of per-table meshes."""
        lib = _lib.load()
        if isinstance(values, (list, tuple)):
            values = np.concatenate([np.asarray(v, np.float64).ravel() for v in values])
        if _is_cuda_tensor(values):
            torch = _torch()
            v = values.to(torch.float64).contiguous().reshape(-1)
            if v.numel() != int(self.offsets[-1]):
                raise ValueError("expected %d values" % int(self.offsets[-1]))
            _lib.check(lib.intp_batch_build(self._h, C.c_void_p(v.data_ptr()), 1, _stream_ptr(stream)))
            self._kept_values = v
        else:
            v = np.ascontiguousarray(np.asarray(values, np.float64).ravel())
            if v.size != int(self.offsets[-1]):
                raise ValueError("expected %d values" % int(self.offsets[-1]))
            _lib.check(lib.intp_batch_build(self._h, v.ctypes.data, 0, _stream_ptr(stream)))
            _lib.check(lib.intp_stream_synchronize(_stream_ptr(stream)))

    def set_schedule(self, persistent=False, contig_rows=32, strided_rows=32):
        """Schedule of the line solves (intp_batch_set_schedule); results do
        not depend on it."""
        sc = _lib.BatchSchedule(int(bool(persistent)), int(contig_rows), int(strided_rows), 0, 0.0)
        _lib.check(_lib.load().intp_batch_set_schedule(self._h, C.byref(sc)))

    def schedule(self):
        sc = _lib.BatchSchedule()
        _lib.check(_lib.load().intp_batch_get_schedule(self._h, C.byref(sc)))
        return sc.as_dict()

    def autotune(self, values, stream=None):
        """Times a build under each candidate schedule (intp_batch_autotune),
        keeps the fastest and leaves the batch built; returns the choice."""
        lib = _lib.load()
        sc = _lib.BatchSchedule()
        if _is_cuda_tensor(values):
            torch = _torch()
            v = values.to(torch.float64).contiguous().reshape(-1)
            _lib.check(lib.intp_batch_autotune(self._h, C.c_void_p(v.data_ptr()), 1, _stream_ptr(stream),
                                               C.byref(sc)))
        else:
            v = np.ascontiguousarray(np.asarray(values, np.float64).ravel())
            _lib.check(lib.intp_batch_autotune(self._h, v.ctypes.data, 0, _stream_ptr(stream), C.byref(sc)))
        return sc.as_dict()

    def control_points(self, i):
        out = np.zeros(self.sizes[i])
        _lib.check(_lib.load().intp_batch_get_control_points(self._h, i, out.ctypes.data))
        shape = list(self.dims[i]) + ([self.channels[i]] if self.channels[i] > 1 else [])
        return out.reshape(shape)

    def evaluate(self, coords, point_offsets, derivs=None, out=None, out_dtype=None, stream=None):
        """Evaluates table i at its points point_offsets[i] .. point_offsets[i+1]-1.
        `coords`: CUDA tensor of every table's points in table order (dim_i
        doubles per point). `derivs`: K rows of up to 4 derivative orders (a
        table of dimension D uses the first D). Returns a (points x K) CUDA
        tensor; a batch with vector-valued tables returns one flat tensor in
        which table i's outputs (its points x K x C_i) follow those of the
        tables before it (`output_views` splits it)."""
        torch = _torch()
        lib = _lib.load()
        po = np.ascontiguousarray(np.asarray(point_offsets, np.int64))
        if po.size != self.ntables + 1:
            raise ValueError("point_offsets needs ntables + 1 entries")
        if out_dtype is None:
            out_dtype = "f32" if self.precision == "mixed" else "f64"
        od = _lib.F32 if out_dtype == "f32" else _lib.F64
        if derivs is None:
            kp, K, karr = None, 1, None
        else:
            d = np.asarray(derivs, np.int32)
            d = d.reshape(-1, d.shape[-1])
            karr = np.zeros((d.shape[0], _lib.MAX_DIM), np.int32)
            karr[:, :d.shape[1]] = d
            K = karr.shape[0]
            kp = karr.ctypes.data
        x = coords.to(torch.float64).contiguous().reshape(-1)
        npts = int(po[-1])
        if out is None:
            dt = torch.float32 if od == _lib.F32 else torch.float64
            if max(self.channels) == 1:
                out = torch.empty((npts, K), dtype=dt, device=x.device)
            else:
                n = np.diff(po)
                out = torch.empty(int(np.sum(n * K * np.asarray(self.channels))), dtype=dt, device=x.device)
        _lib.check(lib.intp_batch_eval(self._h, C.c_void_p(x.data_ptr()), po.ctypes.data, kp, K,
                                       C.c_void_p(out.data_ptr()), od, _stream_ptr(stream)))
        return out

    def graph(self, values, coords, point_offsets, derivs=None, out=None, out_dtype=None):
        """A CUDA graph of one build from `values` and one evaluation of
        `coords` into `out` (CUDA tensors; intp_batch_graph_create). Returns a
        BatchGraph whose launch() replays both, reading the tensors' contents
        at each launch; `out` (allocated here when None) is its `out`."""
        torch = _torch()
        lib = _lib.load()
        po = np.ascontiguousarray(np.asarray(point_offsets, np.int64))
        if po.size != self.ntables + 1:
            raise ValueError("point_offsets needs ntables + 1 entries")
        if not (_is_cuda_tensor(values) and _is_cuda_tensor(coords)):
            raise ValueError("graph buffers are CUDA tensors")
        if values.dtype != torch.float64 or not values.is_contiguous() or values.numel() != int(self.offsets[-1]):
            raise ValueError("values: %d contiguous float64 values" % int(self.offsets[-1]))
        if coords.dtype != torch.float64 or not coords.is_contiguous():
            raise ValueError("coords: contiguous float64")
        if out_dtype is None:
            out_dtype = "f32" if self.precision == "mixed" else "f64"
        od = _lib.F32 if out_dtype == "f32" else _lib.F64
        if derivs is None:
            kp, K, karr = None, 1, None
        else:
            d = np.asarray(derivs, np.int32)
            d = d.reshape(-1, d.shape[-1])
            karr = np.zeros((d.shape[0], _lib.MAX_DIM), np.int32)
            karr[:, :d.shape[1]] = d
            K = karr.shape[0]
            kp = karr.ctypes.data
        if out is None:
            dt = torch.float32 if od == _lib.F32 else torch.float64
            n = np.diff(po)
            out = torch.empty(int(np.sum(n * K * np.asarray(self.channels))), dtype=dt, device=coords.device)
        h = C.c_void_p()
        _lib.check(lib.intp_batch_graph_create(self._h, C.c_void_p(values.data_ptr()), C.c_void_p(coords.data_ptr()),
                                               po.ctypes.data, kp, K, C.c_void_p(out.data_ptr()), od, C.byref(h)))
        return BatchGraph(h, self, (values, coords, out))

    def output_views(self, out, point_offsets, K=1):
        """Table i's outputs as a (points x K) view, or (points x K x C) for a
        vector-valued table, of an `evaluate` result."""
        po = np.asarray(point_offsets, np.int64)
        flat = out.reshape(-1)
        views, e = [], 0
        for i in range(self.ntables):
            n, c = int(po[i + 1] - po[i]), self.channels[i]
            v = flat[e:e + n * K * c]
            views.append(v.reshape(n, K) if c == 1 else v.reshape(n, K, c))
            e += n * K * c
        return views


class BatchGraph:
    """A captured build + evaluation of a TableBatch (TableBatch.graph)."""

    def __init__(self, handle, batch, buffers):
        self._h = handle
        self._batch = batch  # the graph holds the batch's pointers
        self._buffers = buffers
        self.out = buffers[2]

    def launch(self, stream=None):
        _lib.check(_lib.load().intp_batch_graph_launch(self._h, _stream_ptr(stream)))
        return self.out

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.load().intp_batch_graph_destroy(h)
            self._h = None

    def __del__(self):
        self.close()


class Server:
    """Serving loop (intp_server_*): tables stay resident on the device, build
    and evaluate requests run with continuous batching under a memory budget.

    Submissions return request ids at once; `wait` blocks for one. Buffers
    given to a submission (values, points, outputs) must stay alive and
    unchanged until its wait returns; pinned host tensors or CUDA tensors let
    the copies overlap. Table states: "queued", "resident", "gone" (evicted or
    released), "failed".
    """

    STATES = {0: "queued", 1: "resident", 2: "gone", 3: "failed"}

    def __init__(self, memory_budget=0, slots=0, max_batch_points=0):
        lib = _lib.load()
        cfg = _lib.ServerConfig()
        cfg.memory_budget = int(memory_budget)
        cfg.slots = int(slots)
        cfg.max_batch_points = int(max_batch_points)
        h = C.c_void_p()
        _lib.check(lib.intp_server_create(C.byref(cfg), C.byref(h)))
        self._h = h
        self._keep = {}

    def close(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.load().intp_server_destroy(h)
            self._h = None
        self._keep = {}

    def __del__(self):
        self.close()

    @staticmethod
    def _ptr(x):
        if _is_cuda_tensor(x) or (_torch() is not None and isinstance(x, _torch().Tensor)):
            return C.c_void_p(x.data_ptr())
        return C.c_void_p(x.ctypes.data)

    def submit_build(self, order, periodicity, values, *x_ranges, precision="mixed", refine_steps=-1,
                     vector=False):
        """Queues a table build from `values` (mesh, host array or tensor);
        returns (table_id, request_id). vector=True: the last axis of `values`
        holds the C components of a vector-valued table, whose evaluations
        return C values per output (N x K x C)."""
        dims = list(values.shape)
        channels = 1
        if vector:
            channels = dims[-1]
            dims = dims[:-1]
        desc, keep, _, _ = _make_desc(order, periodicity, dims, x_ranges, precision, refine_steps, channels)
        tid, rid = C.c_int64(), C.c_int64()
        _lib.check(_lib.load().intp_server_submit_build(self._h, C.byref(desc), self._ptr(values),
                                                       C.byref(tid), C.byref(rid)))
        self._keep[rid.value] = (values, keep)
        return tid.value, rid.value

    def submit_eval(self, table_id, points, out, derivs=None, out_dtype="f32"):
        """Queues an evaluation of `points` (N x D) into `out` (N x K, or
        N x K x C for a C-channel table); returns the request id."""
        od = _lib.F32 if out_dtype == "f32" else _lib.F64
        if derivs is None:
            kp, K, karr = None, 1, None
        else:
            karr = np.ascontiguousarray(np.asarray(derivs, np.int32))
            K = karr.shape[0]
            kp = karr.ctypes.data
        rid = C.c_int64()
        _lib.check(_lib.load().intp_server_submit_eval(self._h, int(table_id), self._ptr(points),
                                                      int(points.shape[0]), kp, K, self._ptr(out), od,
                                                      C.byref(rid)))
        self._keep[rid.value] = (points, out, karr)
        return rid.value

    def wait(self, request_id, timeout=-1.0):
        """Status of a finished request (0 = OK); raises IntpError on a timeout."""
        st = C.c_int()
        _lib.check(_lib.load().intp_server_wait(self._h, int(request_id), float(timeout), C.byref(st)))
        self._keep.pop(request_id, None)
        return st.value

    def release(self, table_id):
        _lib.check(_lib.load().intp_server_release(self._h, int(table_id)))

    def table_state(self, table_id):
        v = C.c_int32()
        _lib.check(_lib.load().intp_server_table_state(self._h, int(table_id), C.byref(v)))
        return self.STATES[v.value]

    def stats(self):
        st = _lib.ServerStats()
        _lib.check(_lib.load().intp_server_get_stats(self._h, C.byref(st)))
        return st.as_dict()

    def reset_stats(self):
        _lib.check(_lib.load().intp_server_reset_stats(self._h))
