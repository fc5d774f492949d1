"""Long mesh lines solved a warp per line (solve_line_warp): every lane
warms up from a zero state before its segment, checks bit for bit that it
reached its neighbour's values, and is recomputed from them where it did
not. The control points must equal a serial sweep's bit for bit:

- with the warm-up capped at 0 rows (intp_debug_set_segment_warmup), every
  segment but the first is recomputed from its neighbour's final values,
  which is the serial sweep itself; the default warm-up and a 3-row cap
  (some segments recomputed) must give the same bits, for 1D tables built
  alone (warp path) and batched (warp path for a warp's only line);
- 2D tables of 8 lines of length n: built alone their axis-1 lines take the
  warp path, batched they take the lane-per-line path (several lines per
  warp); both must agree bit for bit;
- the FP64 form stays within 1e-12 of the FP64 oracle.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bsplineinterpolation_gb300 as bi
from bsplineinterpolation_gb300 import _lib
from oracle import oracle
from tests.gpu_util import norm_rel_err

pytestmark = pytest.mark.gpu

SIZES = [128, 129, 1000, 4096, 5003]


def _values(rng, n, periodic):
    L = n if periodic else n - 1
    x = np.arange(n, dtype=np.float64)
    f = np.zeros(n)
    for k in range(1, 9):
        f += rng.normal(0.0, 1.0 / k) * np.cos(2 * np.pi * k * x / L + rng.uniform(0, 2 * np.pi))
    return f


def _specs_1d(orders):
    rng = np.random.default_rng(7)
    specs, vals = [], []
    for order in orders:
        for periodic in (False, True):
            for n in SIZES:
                specs.append((order, [periodic], [n], [(0.0, float(n))]))
                vals.append(_values(rng, n, periodic))
    return specs, vals


def _build(specs, vals, precision, cap):
    lib = _lib.load()
    _lib.check(lib.intp_debug_set_segment_warmup(cap))
    try:
        b = bi.TableBatch(specs, precision=precision)
        b.build(vals)
        singles = []
        for (order, per, dims, ranges), v in zip(specs, vals):
            mesh = torch.tensor(np.asarray(v).reshape(dims), device="cuda")
            f = bi.InterpolationFunction(order, per, mesh, *ranges, precision=precision)
            singles.append(f.control_points())
        return [b.control_points(i) for i in range(len(specs))], singles
    finally:
        _lib.check(lib.intp_debug_set_segment_warmup(-1))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_long_lines_equal_under_any_warmup(precision):
    specs, vals = _specs_1d([1, 2, 3, 4, 5, 6, 7])
    serial_b, serial_s = _build(specs, vals, precision, 0)
    for cap in (-1, 3):
        got_b, got_s = _build(specs, vals, precision, cap)
        for i, spec in enumerate(specs):
            assert np.array_equal(got_b[i], serial_b[i]), (cap, spec[0], spec[1], spec[2])
            assert np.array_equal(got_s[i], serial_s[i]), (cap, spec[0], spec[1], spec[2])
    for i, ((order, per, dims, ranges), v) in enumerate(zip(specs, vals)):
        assert np.array_equal(serial_b[i], serial_s[i]), (order, per, dims)
        if precision == "fp64":
            s = oracle.Spline(1, order, per, dims, [0.0], [float(dims[0])])
            s.interpolate(v)
            assert norm_rel_err(serial_b[i].ravel(), s.control_points().ravel()) < 1e-12, (order, per, dims)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_warp_path_equals_lane_path(precision):
    rng = np.random.default_rng(11)
    specs, vals = [], []
    for order in (3, 5):
        for periodic in (False, True):
            for n in (128, 129, 1000, 2000):
                specs.append((order, [False, periodic], [8, n], [(0.0, 8.0), (0.0, float(n))]))
                vals.append(np.stack([_values(rng, n, periodic) for _ in range(8)]))
    got_b, got_s = _build(specs, vals, precision, -1)
    for i, spec in enumerate(specs):
        assert np.array_equal(got_b[i], got_s[i]), (spec[0], spec[1], spec[2])
