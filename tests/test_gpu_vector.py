"""Vector-valued tables (the reference's InterpolationFunction<T, D, O> with a
vector type T): C channels share the knots, the band factors and, per
query, the basis weights.

A C-channel table must give exactly what C scalar tables built from the
separate channels give: the line solves run channel by channel with the same
substitution code, and evaluation contracts each channel with the same
weights in the same order.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bsplineinterpolation_gb300 as bi
from oracle import oracle
from tests.gpu_util import norm_rel_err

pytestmark = pytest.mark.gpu


def _field(rng, dims, C):
    axes = np.meshgrid(*[np.linspace(0.0, 1.0, n) for n in dims], indexing="ij")
    out = np.empty(list(dims) + [C])
    for c in range(C):
        f = np.ones(dims)
        for a in axes:
            f = f * np.cos(rng.uniform(1, 5) * a + rng.uniform(0, 6.28))
        out[..., c] = f + 1e-3 * rng.normal(size=dims)
    return out


CASES = [  # (order, periodicity, dims, channels)
    (3, [False, False], [40, 36], 3),
    (5, [True, False], [32, 30], 2),
    (3, [False, False, False], [16, 18, 20], 4),
    (4, [True], [50], 2),
]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", CASES, ids=lambda c: "o%d_d%d_c%d" % (c[0], len(c[2]), c[3]))
def test_vector_table_equals_scalar_tables(case, precision):
    order, per, dims, C = case
    rng = np.random.default_rng(7)
    vals = _field(rng, dims, C)
    ranges = [(0.0, 1.0)] * len(dims)
    f = bi.InterpolationFunction(order, per, vals, *ranges, precision=precision, vector=True)
    assert f.channels == C
    pts = rng.uniform(-0.05, 1.05, (3000, len(dims)))
    derivs = np.zeros((2, len(dims)), np.int32)
    derivs[1, -1] = 1
    got = f.evaluate(torch.tensor(pts, device="cuda"), derivs=derivs).double().cpu().numpy()
    assert got.shape == (3000, 2, C)
    ctrl = f.control_points()
    assert ctrl.shape == tuple(dims) + (C,)
    for c in range(C):
        s = bi.InterpolationFunction(order, per, np.ascontiguousarray(vals[..., c]), *ranges, precision=precision)
        assert np.array_equal(ctrl[..., c], s.control_points())
        want = s.evaluate(torch.tensor(pts, device="cuda"), derivs=derivs).double().cpu().numpy()
        assert np.array_equal(got[:, :, c], want), c


@pytest.mark.parametrize("case", CASES, ids=lambda c: "o%d_d%d_c%d" % (c[0], len(c[2]), c[3]))
def test_vector_table_fp64_matches_reference(case):
    order, per, dims, C = case
    rng = np.random.default_rng(11)
    vals = _field(rng, dims, C)
    D = len(dims)
    f = bi.InterpolationFunction(order, per, vals, *[(0.0, 1.0)] * D, vector=True)
    pts = rng.uniform(0.0, 1.0, (2000, D))
    got = f.evaluate(pts)  # host buffers
    for c in range(C):
        ref = oracle.Spline(D, order, per, dims, [0.0] * D, [1.0] * D).interpolate(vals[..., c])
        assert norm_rel_err(got[:, 0, c], ref.eval(pts)) < 1e-12


def test_control_points_round_trip():
    rng = np.random.default_rng(3)
    vals = _field(rng, [24, 20], 3)
    f = bi.InterpolationFunction(3, [False, False], vals, (0.0, 1.0), (0.0, 1.0), vector=True)
    ctrl = f.control_points()
    t = bi.InterpolationFunctionTemplate(3, [False, False], [24, 20], (0.0, 1.0), (0.0, 1.0), channels=3)
    g = t.interpolate(vals)
    assert np.array_equal(g.control_points(), ctrl)
    from bsplineinterpolation_gb300 import _lib
    lib = _lib.load()
    flipped = np.ascontiguousarray(ctrl[::-1, ::-1])  # kept alive across the call
    _lib.check(lib.intp_table_set_control_points(g._h, flipped.ctypes.data))
    assert np.array_equal(g.control_points(), flipped)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_points_on_a_circle(precision):
    """The reference's own vector test (test/src/interpolation-test.cpp,
    interpolation on vector): 31 points on the unit circle as a periodic
    1D cubic of 2-vectors; sampled at 1024 angles the magnitude stays within
    1e-5 of 1 on average."""
    n = 31
    theta = 2 * np.pi * np.arange(n) / n
    pts = np.stack([np.cos(theta), np.sin(theta)], axis=1)
    circle = bi.InterpolationFunction1D(3, pts, periodic=True, precision=precision)
    assert circle.channels == 2
    s = 2 * np.pi * np.arange(1024) / 1024
    v = circle.evaluate(s.reshape(-1, 1)).astype(np.float64)[:, 0, :]
    err = np.mean(np.abs(np.hypot(v[:, 0], v[:, 1]) - 1.0))
    assert err < 1e-5
    one = circle(0.5)
    assert one.shape == (2,)


@pytest.mark.parametrize("case", [(3, [False, True, False], [40, 36, 32], 2), (5, [True, True], [64, 60], 3)],
                         ids=["o3_d3_c2", "o5_d2_c3"])
def test_vector_table_binned_path(case):
    """2^19 points send a mixed vector-valued table down the binned path,
    each channel's tiles staged in turn: every channel equals the scalar
    table of that channel on the same path bit for bit (value and d/dx), and
    the oracle's scalar table within 1e-6."""
    order, per, dims, C = case
    rng = np.random.default_rng(17)
    vals = _field(rng, dims, C)
    D = len(dims)
    ranges = [(0.0, 1.0)] * D
    f = bi.InterpolationFunction(order, per, vals, *ranges, precision="mixed", vector=True)
    n = 1 << 19
    pts = rng.uniform(0.0, 1.0, (n, D))
    x = torch.tensor(pts, device="cuda")
    derivs = np.zeros((2, D), np.int32)
    derivs[1, 0] = 1
    got = f.evaluate(x, derivs=derivs).double().cpu().numpy()
    assert got.shape == (n, 2, C)
    for c in range(C):
        s = bi.InterpolationFunction(order, per, np.ascontiguousarray(vals[..., c]), *ranges, precision="mixed")
        want = s.evaluate(x, derivs=derivs).double().cpu().numpy()
        assert np.array_equal(got[:, :, c], want), c
        ref = oracle.Spline(D, order, per, dims, [0.0] * D, [1.0] * D).interpolate(vals[..., c])
        assert norm_rel_err(got[:20000, 0, c], ref.eval(pts[:20000])) < 1e-6, c
