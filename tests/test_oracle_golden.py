"""The CPU oracle against the known-answer vectors of the reference's own tests
(test/src/interpolation-test.cpp, test/src/bspline-test.cpp) at the tolerances
those tests use, and against the band-solver residual test
(test/src/band-matrix-and-solver-test.cpp)."""
import numpy as np
import pytest

from oracle import oracle
from tests.golden_cases import expected, full_f, reference_cases, rel_err

CASES = reference_cases()
F13 = full_f(CASES)


def _spline(case):
    D = case["dim"]
    ranges = case.get("ranges") or [None] * D
    coords = case.get("coords") or [None] * D
    lo = [r[0] if r else 0.0 for r in ranges]
    hi = [r[1] if r else 0.0 for r in ranges]
    s = oracle.Spline(D, case["order"], case["periodic"], case["sizes"], lo, hi, coords)
    s.interpolate(np.asarray(case["values"]).reshape(case["sizes"]))
    return s


@pytest.mark.parametrize("case", [c for c in CASES if c["kind"] == "interp"],
                         ids=lambda c: c["name"])
def test_interpolation_golden(case):
    s = _spline(case)
    pts = np.asarray(case["points"], np.float64).reshape(-1, case["dim"])
    if case.get("derivs"):
        got = s.derivative(pts, case["derivs"])[:, 0]
    else:
        got = s.eval(pts)
    want = expected(case, F13)
    if case["name"].endswith("extrapolation") or case["name"].endswith("wrap"):
        assert np.max(np.abs(got - want)) < case["tol"], case["cite"]
    else:
        assert rel_err(got, want) < case["tol"], case["cite"]


@pytest.mark.parametrize("case", [c for c in CASES if c["kind"] == "bspline"],
                         ids=lambda c: c["name"])
def test_bspline_golden(case):
    s = oracle.Spline.from_knots(case["dim"], case["order"], case["periodic"], case["ncp"],
                                 case["knots"], case["ctrl"])
    pts = np.asarray(case["points"], np.float64).reshape(-1, case["dim"])
    if case.get("derivs"):
        got = s.derivative(pts, case["derivs"])[:, 0]
    else:
        got = s.eval(pts)
    assert rel_err(got, case["expected"]) < case["tol"], case["cite"]


def test_domain_error_case():
    case = [c for c in CASES if c["kind"] == "domain_error"][0]
    s = _spline(case)
    assert not s.in_range(case["points"])
    assert s.in_range([1.0, 1.0])


def _band_cases(n):
    """The matrices of test/src/band-matrix-and-solver-test.cpp:54-106."""
    lap = np.zeros((n, n))
    for i in range(n):
        lap[i, i] = -2
        if i > 0:
            lap[i, i - 1] = 1
        if i < n - 1:
            lap[i, i + 1] = 1
    yield "laplacian", lap, 1, 1, False
    m1 = np.zeros((n, n))
    for i in range(n):
        m1[i, i] = 3 / 4
        m1[i, (i + n - 1) % n] = 1 / 8
        m1[i, (i + 1) % n] = 1 / 8
    yield "cyclic_o2", m1, 1, 1, True
    m2 = np.zeros((n, n))
    for i in range(n):
        m2[i, i] = 115 / 192
        m2[i, (i + n - 1) % n] = 19 / 96
        m2[i, (i + 1) % n] = 19 / 96
        m2[i, (i + n - 2) % n] = 1 / 384
        m2[i, (i + 2) % n] = 1 / 384
    yield "cyclic_o4", m2, 2, 2, True
    m3 = np.zeros((n, n))
    for i in range(n):
        m3[i, (i + n - 1) % n] = 2889 / 16000
        m3[i, i] = 1701 / 3200
        m3[i, (i + 1) % n] = 33 / 128
        m3[i, (i + 2) % n] = 729 / 20000
        m3[i, (i + 3) % n] = 9 / 20000
    yield "cyclic_1_3", m3, 1, 3, True


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_band_solver_residual(seed):
    n = 64
    b = np.random.default_rng(seed).uniform(-1, 1, n)
    for name, a, p, q, cyc in _band_cases(n):
        x = oracle.band_solve_dense(a, b, p, q, cyc)
        assert rel_err(a @ x, b) < 1e-10, name
