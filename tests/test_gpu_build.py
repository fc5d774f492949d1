"""The mixed form's control-point build on 3D tables.

The refinement's residual r = F - (A_0 x A_1 x A_2) c runs as one fused
kernel (residual3d.cu) that marches along axis 0 with the intermediate passes
in shared memory; the per-axis pass kernels remain selectable with
INTP_GB300_RESIDUAL=passes. Both apply the same Dot2 accumulations in the
same order, so the refined control points must agree bit for bit. The last
correction solve adds its solution to the control points in its back sweep;
the control points are checked against the oracle (the reference algorithm
in FP64) as well."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bsplineinterpolation_gb300 as bi
from oracle import oracle
from tests.gpu_util import norm_rel_err

pytestmark = pytest.mark.gpu


def _build(order, periodic, values, mode, vector=False):
    old = os.environ.get("INTP_GB300_RESIDUAL")
    try:
        if mode == "passes":
            os.environ["INTP_GB300_RESIDUAL"] = "passes"
        else:
            os.environ.pop("INTP_GB300_RESIDUAL", None)
        f = bi.InterpolationFunction(order, periodic, torch.tensor(values, device="cuda"), *[(0.0, 1.0)] * 3,
                                     precision="mixed", vector=vector)
        torch.cuda.synchronize()
        return f.control_points()
    finally:
        if old is None:
            os.environ.pop("INTP_GB300_RESIDUAL", None)
        else:
            os.environ["INTP_GB300_RESIDUAL"] = old


CASES = [
    # order, periodic, sizes
    (3, [False, False, False], (64, 48, 40)),
    (3, [True, False, True], (33, 40, 70)),
    (5, [True, True, True], (24, 30, 36)),
    (1, [False, True, False], (17, 5, 90)),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: "o%d_%s_%s" % (c[0], "".join("p" if p else "n" for p in c[1]),
                                                                     "x".join(map(str, c[2]))))
def test_fused_residual_matches_per_axis_passes(case):
    order, periodic, sizes = case
    rng = np.random.default_rng(sum(sizes) + order)
    v = rng.normal(size=sizes)
    fused = _build(order, periodic, v, "fused")
    passes = _build(order, periodic, v, "passes")
    assert np.array_equal(fused, passes)
    ref = oracle.Spline(3, order, periodic, list(sizes), [0.0] * 3, [1.0] * 3).interpolate(v)
    assert norm_rel_err(fused.ravel(), ref.control_points().ravel()) < 1e-11


def test_fused_residual_vector_table():
    rng = np.random.default_rng(5)
    v = rng.normal(size=(20, 24, 28, 2))
    fused = _build(3, [False] * 3, v, "fused", vector=True)
    passes = _build(3, [False] * 3, v, "passes", vector=True)
    assert np.array_equal(fused, passes)
