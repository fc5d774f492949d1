"""The benchmark workloads' own shapes, against the oracle (the C restatement
of the reference, pinned bit-exact to the reference's build).

- Plain method: 2D, order 3, FP64, non-periodic, 64 x 64 on [0,1] x [0,2],
  z = sin(3x) cos(2y) + N(0, 0.01^2), 1e5 uniform points: the FP64 form
  matches the reference to 1e-12 (relative to max |f|), spans bit-exact.
- Periodic high order: 2D, order 7, periodic in both axes, 512 x 512 of a
  sum of 16 random sinusoids (integer wavenumbers 1..20). Value, first and
  second derivatives: the FP64 form to 1e-12; the mixed form (cyclic solve
  in double-word arithmetic, FP32 weights, the precise contraction for
  second derivatives) to 1e-6 on every output.
- 3D cubic (the headline workload at 64^3): FP64 to 1e-12; the mixed form's
  value and d/dx within 1e-6 of max |.|, its control points (double-words
  from the double-word solve) within 1e-11 of the FP64 form's.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bsplineinterpolation_gb300 as bi
from oracle import oracle
from tests.gpu_util import norm_rel_err

pytestmark = pytest.mark.gpu


def test_plain_2d_cubic_fp64_matches_reference():
    rng = np.random.default_rng(20261203)
    x = np.linspace(0.0, 1.0, 64)
    y = np.linspace(0.0, 2.0, 64)
    z = np.sin(3 * x)[:, None] * np.cos(2 * y)[None, :] + rng.normal(0.0, 0.01, (64, 64))
    pts = rng.uniform([0.0, 0.0], [1.0, 2.0], (100_000, 2))
    ref = oracle.Spline(2, 3, [False, False], [64, 64], [0.0, 0.0], [1.0, 2.0]).interpolate(z)
    f = bi.InterpolationFunction(3, [False, False], torch.tensor(z, device="cuda"), (0.0, 1.0), (0.0, 2.0))
    p = torch.tensor(pts, device="cuda")
    got = f.evaluate(p).cpu().numpy()[:, 0]
    assert norm_rel_err(got, ref.eval(pts)) < 1e-12
    cells, _ = f.locate(p)
    want_cells, _ = ref.locate(pts)
    assert np.array_equal(cells.cpu().numpy(), want_cells)
    assert norm_rel_err(f.control_points().ravel(), ref.control_points().ravel()) < 1e-12


def _sinusoids(n, rng):
    g = np.arange(n) * (2 * np.pi / n)  # one period over the axis range [0, 2 pi)
    X, Y = np.meshgrid(g, g, indexing="ij")
    f = np.zeros((n, n))
    for _ in range(16):
        kx, ky = rng.integers(1, 21, 2)
        f += np.sin(kx * X + ky * Y + rng.uniform(0, 2 * np.pi))
    return f


DERIVS_2ND = [[0, 0], [1, 0], [0, 1], [2, 0], [1, 1], [0, 2]]


@pytest.fixture(scope="module")
def periodic_o7():
    rng = np.random.default_rng(20261203 + 3)
    n = 512
    f = _sinusoids(n, rng)
    rng_ = (0.0, 2 * np.pi)
    ref = oracle.Spline(2, 7, [True, True], [n, n], [0.0, 0.0], [2 * np.pi] * 2).interpolate(f)
    pts = rng.uniform(0.0, 2 * np.pi, (20_000, 2))
    want = ref.derivative(pts, DERIVS_2ND)
    kappa = float(np.max(np.abs(ref.control_points())) / np.max(np.abs(f)))
    return f, rng_, pts, want, kappa


def test_periodic_order7_fp64_matches_reference(periodic_o7):
    f, rng_, pts, want, _ = periodic_o7
    t = bi.InterpolationFunction(7, [True, True], torch.tensor(f, device="cuda"), rng_, rng_)
    got = t.evaluate(torch.tensor(pts, device="cuda"), derivs=DERIVS_2ND).cpu().numpy()
    for k in range(len(DERIVS_2ND)):
        assert norm_rel_err(got[:, k], want[:, k]) < 1e-12, DERIVS_2ND[k]


def test_periodic_order7_mixed_within_stated_error(periodic_o7):
    """Mixed form on the periodic order-7 table: the cyclic solve runs in
    double-word arithmetic (control points near 1e-13 of the FP64 form's). A
    request with second derivatives takes
    the precise contraction (operands relative to each query's central
    control point in double-float, recursion-based derivative weights,
    compensated sums). Every output, values through second derivatives,
    within 1e-6 of its max magnitude."""
    f, rng_, pts, want, _ = periodic_o7
    t = bi.InterpolationFunction(7, [True, True], torch.tensor(f, device="cuda"), rng_, rng_, precision="mixed")
    got = t.evaluate(torch.tensor(pts, device="cuda"), derivs=DERIVS_2ND).double().cpu().numpy()
    tol = [1e-6] * 6
    for k in range(len(DERIVS_2ND)):
        assert norm_rel_err(got[:, k], want[:, k]) < tol[k], (DERIVS_2ND[k], norm_rel_err(got[:, k], want[:, k]))


def test_cube_3d_cubic_both_forms():
    rng = np.random.default_rng(20261203 + 1)
    n = 64
    g = np.linspace(-1.0, 1.0, n)
    X, Y, Zc = np.meshgrid(g, g, g, indexing="ij")
    v = np.exp(-(X * X + Y * Y + Zc * Zc)) * np.cos(4 * X) + rng.normal(0.0, 1e-3, (n, n, n))
    pts = rng.uniform(-1.0, 1.0, (400_000, 3))
    ref = oracle.Spline(3, 3, [False] * 3, [n] * 3, [-1.0] * 3, [1.0] * 3).interpolate(v)
    want = ref.derivative(pts, [[0, 0, 0], [1, 0, 0]])
    p = torch.tensor(pts, device="cuda")
    f64 = bi.InterpolationFunction(3, [False] * 3, torch.tensor(v, device="cuda"), (-1.0, 1.0), (-1.0, 1.0),
                                   (-1.0, 1.0))
    got = f64.evaluate(p, derivs=[[0, 0, 0], [1, 0, 0]]).cpu().numpy()
    assert norm_rel_err(got, want) < 1e-12
    mix = bi.InterpolationFunction(3, [False] * 3, torch.tensor(v, device="cuda"), (-1.0, 1.0), (-1.0, 1.0),
                                   (-1.0, 1.0), precision="mixed")
    got = mix.evaluate(p, derivs=[[0, 0, 0], [1, 0, 0]]).double().cpu().numpy()
    assert norm_rel_err(got[:, 0], want[:, 0]) < 1e-6
    assert norm_rel_err(got[:, 1], want[:, 1]) < 1e-6
    assert norm_rel_err(mix.control_points().ravel(), f64.control_points().ravel()) < 1e-11
