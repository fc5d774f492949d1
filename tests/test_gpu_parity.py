"""CUDA path against the golden fixtures and the oracle (runs on a GPU).

FP64 form: the reference's own tolerances on its known-answer vectors
(1e-14 for test/src/interpolation-test.cpp, 1e-15 for bspline-test.cpp
cases evaluated through the interpolation API), 1e-12 normwise against the
reference's outputs, and bit-exact knot spans and periodic-wrapped
coordinates."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bsplineinterpolation_gb300 as bi
from tests.golden_cases import expected, full_f, ref_outputs, reference_cases, rel_err
from tests.gpu_util import norm_rel_err

pytestmark = pytest.mark.gpu

CASES = reference_cases()
F13 = full_f(CASES)
Z, INDEX = ref_outputs()


def _ranges(case):
    D = case["dim"]
    ranges = case.get("ranges") or [None] * D
    coords = case.get("coords") or [None] * D
    return [tuple(ranges[d]) if coords[d] is None else coords[d] for d in range(D)]


@pytest.mark.parametrize("case", [c for c in CASES if c["kind"] == "interp"], ids=lambda c: c["name"])
def test_golden_interpolation_fp64(case):
    mesh = np.asarray(case["values"], np.float64).reshape(case["sizes"])
    f = bi.InterpolationFunction(case["order"], case["periodic"], torch.tensor(mesh, device="cuda"),
                                 *_ranges(case))
    pts = torch.tensor(np.asarray(case["points"], np.float64).reshape(-1, case["dim"]), device="cuda")
    if case.get("derivs"):
        got = f.evaluate(pts, derivs=case["derivs"]).cpu().numpy()[:, 0]
    else:
        got = f.evaluate(pts).cpu().numpy()[:, 0]
    want = expected(case, F13)
    if case["name"].endswith(("extrapolation", "wrap")):
        assert np.max(np.abs(got - want)) < case["tol"], case["cite"]
    else:
        assert rel_err(got, want) < case["tol"], case["cite"]


def test_golden_domain_error():
    case = [c for c in CASES if c["kind"] == "domain_error"][0]
    mesh = np.asarray(case["values"], np.float64).reshape(case["sizes"])
    f = bi.InterpolationFunction(case["order"], case["periodic"], mesh, *_ranges(case))
    with pytest.raises(bi.IntpDomainError):
        f.at(*case["points"])
    f.at(1.0, 1.0)


def _table(meta, precision="fp64", refine_steps=-1):
    name = meta["name"]
    D = meta["dim"]
    ranges = [Z[name + "/coords%d" % d] if meta["nonuniform"][d] else (meta["lo"][d], meta["hi"][d])
              for d in range(D)]
    mesh = Z[name + "/values"].reshape(meta["sizes"])
    return bi.InterpolationFunction(meta["order"], meta["periodic"], torch.tensor(mesh, device="cuda"),
                                    *ranges, precision=precision, refine_steps=refine_steps)


@pytest.mark.parametrize("meta", INDEX, ids=lambda m: m["name"])
def test_reference_outputs_fp64(meta):
    name = meta["name"]
    f = _table(meta)
    for d in range(meta["dim"]):
        assert np.array_equal(f.knots(d), Z[name + "/knots%d" % d])
        assert f.range(d) == tuple(Z[name + "/range"][d])
    ctrl = f.control_points().ravel()
    assert norm_rel_err(ctrl, Z[name + "/ctrl"]) < 1e-12
    pts = torch.tensor(Z[name + "/points"], device="cuda")
    cells, wrapped = f.locate(pts)
    assert np.array_equal(cells.cpu().numpy(), Z[name + "/cells"])
    assert np.array_equal(wrapped.cpu().numpy(), Z[name + "/wrapped"])
    val = f.evaluate(pts).cpu().numpy()[:, 0]
    assert norm_rel_err(val, Z[name + "/value"]) < 1e-12
    der = f.evaluate(pts, derivs=Z[name + "/derivs"]).cpu().numpy()
    assert norm_rel_err(der, Z[name + "/deriv"]) < 1e-12


def _in_domain(meta, pts):
    rng_ = Z[meta["name"] + "/range"]
    ok = np.ones(pts.shape[0], bool)
    for d in range(meta["dim"]):
        if not meta["periodic"][d]:
            ok &= (pts[:, d] >= rng_[d, 0]) & (pts[:, d] <= rng_[d, 1])
    return ok


def mixed_tolerance(ctrl, values):
    """Bound of the mixed form inside the domain: FP32 weights carry ~1e-7
    relative rounding that multiplies every control point of the contraction,
    so the error relative to max|f| is held to 1e-6 * max(1, kappa) with
    kappa = max|c| / max|f| (kappa ~ 1 for smooth data on uniform grids; it
    grows for high orders on rough data and strongly non-uniform knots)."""
    kappa = float(np.max(np.abs(ctrl)) / np.max(np.abs(values)))
    return 1e-6 * max(1.0, kappa)


@pytest.mark.parametrize("meta", INDEX, ids=lambda m: m["name"])
def test_reference_outputs_mixed(meta):
    """Mixed form: spans still bit-exact; values inside the domain within
    mixed_tolerance of the FP64 reference. Extrapolated points (outside a
    non-periodic range) carry FP32's growth of (x - t_c)^O and are held to
    1e3 times that bound."""
    name = meta["name"]
    f = _table(meta, precision="mixed")
    pts_np = Z[name + "/points"]
    pts = torch.tensor(pts_np, device="cuda")
    cells, _ = f.locate(pts)
    assert np.array_equal(cells.cpu().numpy(), Z[name + "/cells"])
    val = f.evaluate(pts).double().cpu().numpy()[:, 0]
    want = Z[name + "/value"]
    inside = _in_domain(meta, pts_np)
    tol = mixed_tolerance(Z[name + "/ctrl"], want[inside])
    assert norm_rel_err(val[inside], want[inside]) < tol
    assert norm_rel_err(val, want) < 1e3 * tol


@pytest.mark.parametrize("meta", [m for m in INDEX if m["name"] in ("plain_2d_o3_64x64", "cube_3d_o3_20",
                                                                    "periodic_2d_o7_48x40")],
                         ids=lambda m: m["name"])
def test_mixed_workload_shapes_within_1e6(meta):
    """The workload-shaped tables (smooth data, uniform grids) meet 1e-6 on
    values with the plain FP32 solve (refine_steps = 0) and with the
    double-word solve (the default)."""
    name = meta["name"]
    pts_np = Z[name + "/points"]
    inside = _in_domain(meta, pts_np)
    want = Z[name + "/value"][inside]
    for steps in (0, 1):
        f = _table(meta, precision="mixed", refine_steps=steps)
        val = f.evaluate(torch.tensor(pts_np, device="cuda")).double().cpu().numpy()[inside, 0]
        assert norm_rel_err(val, want) < 1e-6, steps


@pytest.mark.parametrize("meta", [m for m in INDEX if m["dim"] <= 3], ids=lambda m: m["name"])
def test_binned_spans_match_reference(meta):
    """The binned evaluation path locates queries with its own kernel (exact
    integer knot keys, a 32-bit FP32 hint, the span packed into its sort
    records). Its spans, read back from those records, equal the reference's
    get_knot_iter (BSpline.hpp:125-157) bit for bit on every case: points on
    knots, at both ends of non-periodic ranges, outside them, and wrapped
    around periodic axes."""
    name = meta["name"]
    f = _table(meta, precision="mixed")
    pts = torch.tensor(Z[name + "/points"], device="cuda")
    got = f.locate_binned(pts).cpu().numpy()
    assert np.array_equal(got, Z[name + "/cells"])
    # the same spans in a batch large enough for intp_eval to bin it
    reps = (1 << 18) // pts.shape[0] + 1
    big = pts.repeat(reps, 1)
    got = f.locate_binned(big).cpu().numpy()
    assert np.array_equal(got, np.tile(Z[name + "/cells"], (reps, 1)))
