"""The headline workload at full mesh size against the oracle.

3D, order 3, non-periodic, 256^3 mesh on [-1, 1]^3 of
f = exp(-r^2) cos(4x) + N(0, 1e-3^2); queries drawn by the benchmark's own
generator (half uniform in the cube, half Gaussian with sigma 0.05 around 8
random centres), 1e6 of them; outputs value and d/dx.

- FP64 form: within 1e-12 of the oracle (relative to each output's max
  magnitude), spans bit-exact.
- Mixed form (double-word solve, binned FP32 evaluation): within 1e-6 of
  the oracle, and the binned path's spans
  bit-exact against the oracle's get_knot_iter (BSpline.hpp:125-157).
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bsplineinterpolation_gb300 as bi
from bench import DERIVS, SEED, make_points_np, make_values_np
from oracle import oracle
from tests.gpu_util import norm_rel_err

pytestmark = pytest.mark.gpu

N = 256
NPTS = 1_000_000


@pytest.fixture(scope="module")
def headline():
    rng = np.random.default_rng(SEED)
    vals = make_values_np(N, rng)
    pts = make_points_np(NPTS, rng)
    threads = os.cpu_count() or 1
    ref = oracle.Spline(3, 3, [False] * 3, [N] * 3, [-1.0] * 3, [1.0] * 3)
    ref.interpolate(vals, nthreads=threads)
    want = ref.derivative(pts, DERIVS, nthreads=threads)
    cells, _ = ref.locate(pts)
    return vals, pts, want, cells


def _table(vals, precision):
    return bi.InterpolationFunction(3, [False] * 3, torch.tensor(vals, device="cuda"), (-1.0, 1.0), (-1.0, 1.0),
                                    (-1.0, 1.0), precision=precision)


def test_headline_fp64_matches_oracle(headline):
    vals, pts, want, cells = headline
    f = _table(vals, "fp64")
    p = torch.tensor(pts, device="cuda")
    got = f.evaluate(p, derivs=DERIVS).cpu().numpy()
    for k in range(len(DERIVS)):
        assert norm_rel_err(got[:, k], want[:, k]) < 1e-12, DERIVS[k]
    got_cells, _ = f.locate(p)
    assert np.array_equal(got_cells.cpu().numpy(), cells)


def test_headline_mixed_within_1e6_of_oracle(headline):
    vals, pts, want, cells = headline
    f = _table(vals, "mixed")
    p = torch.tensor(pts, device="cuda")
    got = f.evaluate(p, derivs=DERIVS).double().cpu().numpy()
    for k in range(len(DERIVS)):
        err = norm_rel_err(got[:, k], want[:, k])
        assert err < 1e-6, (DERIVS[k], err)
    assert np.array_equal(f.locate_binned(p).cpu().numpy(), cells)
