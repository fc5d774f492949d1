"""Evaluation proxies (the reference's eval_proxy / pre_calc_coef,
InterpolationTemplate.hpp:145-176, Interpolation.hpp:493-503, BSpline.hpp:
250-296): spans and value weights of a point set computed once and reused for
every function interpolated from one template. Each value equals the
function's own direct evaluation bit for bit (same arithmetic), matches the
oracle at 1e-12 in the FP64 form, and a table with other knots is refused."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bsplineinterpolation_gb300 as bi
from bsplineinterpolation_gb300 import _lib
from oracle import oracle

pytestmark = pytest.mark.gpu


def _meshes(rng, dims, k):
    axes = np.meshgrid(*[np.linspace(0, 1, n) for n in dims], indexing="ij")
    out = []
    for j in range(k):
        f = np.cos((j + 1) * 2.1 * axes[0]) + rng.normal(0, 0.05, dims)
        for a in axes[1:]:
            f = f * np.sin(1.3 * a + j)
        out.append(f)
    return out


CASES = [
    (1, 0, [False], [40]),
    (1, 5, [True], [33]),
    (2, 3, [False, True], [30, 21]),
    (2, 7, [True, True], [25, 26]),
    (3, 3, [True, False, False], [18, 15, 17]),
    (3, 4, [False, False, True], [12, 14, 13]),
]


@pytest.mark.parametrize("dim,order,periodic,dims", CASES)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_proxy_equals_direct_evaluation(dim, order, periodic, dims, precision):
    rng = np.random.default_rng(dim * 10 + order)
    lo, hi = [0.0] * dim, [2.0] * dim
    tmpl = bi.InterpolationFunctionTemplate(order, periodic, dims, *[(0.0, 2.0)] * dim, precision=precision)
    meshes = _meshes(rng, dims, 3)
    funcs = [tmpl.interpolate(torch.tensor(m, device="cuda")) for m in meshes]
    # periodic axes wrap; non-periodic axes extrapolate a little past the range
    pts = rng.uniform(-0.3, 2.3, (20_000, dim))
    dp = torch.tensor(pts, device="cuda")
    proxy = tmpl.eval_proxy(dp)
    got = proxy(*funcs, out_dtype="f64").cpu().numpy()
    for j, f in enumerate(funcs):
        want = f.evaluate(dp, out_dtype="f64").cpu().numpy()[:, 0]
        assert np.array_equal(got[:, j], want), (j, np.max(np.abs(got[:, j] - want)))
    one = proxy(funcs[1], out_dtype="f64").cpu().numpy()
    assert np.array_equal(one, got[:, 1])
    if precision == "fp64":
        for j, m in enumerate(meshes):
            ref = oracle.Spline(dim, order, periodic, dims, lo, hi).interpolate(m).eval(pts)
            err = np.max(np.abs(got[:, j] - ref)) / max(np.max(np.abs(ref)), 1e-300)
            assert err < 1e-12, (j, err)


def test_proxy_refuses_tables_with_other_knots():
    rng = np.random.default_rng(5)
    t1 = bi.InterpolationFunctionTemplate(3, [False, False], [20, 20], (0, 1), (0, 1))
    t2 = bi.InterpolationFunctionTemplate(3, [False, False], [20, 20], (0, 1), (0, 2))
    m = torch.tensor(rng.normal(size=(20, 20)), device="cuda")
    f1, f2 = t1.interpolate(m), t2.interpolate(m)
    proxy = t1.eval_proxy(torch.rand((100, 2), dtype=torch.float64, device="cuda"))
    proxy(f1)
    with pytest.raises(_lib.IntpError):
        proxy(f1, f2)
    fm = bi.InterpolationFunctionTemplate(3, [False, False], [20, 20], (0, 1), (0, 1), precision="mixed").interpolate(m)
    with pytest.raises(_lib.IntpError):
        proxy(fm)


def test_proxy_of_a_function_and_empty_point_set():
    rng = np.random.default_rng(6)
    f = bi.InterpolationFunction(3, [False, False, False], torch.tensor(rng.normal(size=(9, 10, 11)), device="cuda"),
                                 (0, 1), (0, 1), (0, 1))
    pts = torch.rand((5000, 3), dtype=torch.float64, device="cuda")
    assert np.array_equal(f.eval_proxy(pts)(f).cpu().numpy(), f.evaluate(pts).cpu().numpy()[:, 0])
    empty = f.eval_proxy(torch.empty((0, 3), dtype=torch.float64, device="cuda"))
    assert empty(f).shape == (0,)
