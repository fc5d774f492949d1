"""The CPU oracle against outputs of the reference library itself.

ref_outputs.npz was recorded by tests/golden/make_golden.py from the
reference headers compiled in place (oracle/build_ref.sh). The comparison is
bit-exact: the oracle restates the reference's arithmetic operation by
operation and is compiled without FMA contraction."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import oracle
from tests.golden_cases import ref_outputs

Z, INDEX = ref_outputs()


def _spline(meta):
    name = meta["name"]
    D = meta["dim"]
    coords = [Z[name + "/coords%d" % d] if meta["nonuniform"][d] else None for d in range(D)]
    s = oracle.Spline(D, meta["order"], meta["periodic"], meta["sizes"], meta["lo"], meta["hi"],
                      coords)
    s.interpolate(Z[name + "/values"].reshape(meta["sizes"]))
    return s


@pytest.mark.parametrize("meta", INDEX, ids=lambda m: m["name"])
def test_bit_exact_against_reference(meta):
    name = meta["name"]
    s = _spline(meta)
    for d in range(meta["dim"]):
        assert np.array_equal(s.knots(d), Z[name + "/knots%d" % d])
        assert np.array_equal(np.array(s.range(d)), Z[name + "/range"][d])
    assert np.array_equal(s.control_points().ravel(), Z[name + "/ctrl"])
    pts = Z[name + "/points"]
    cells, wrapped = s.locate(pts)
    assert np.array_equal(cells, Z[name + "/cells"])
    assert np.array_equal(wrapped, Z[name + "/wrapped"])
    assert np.array_equal(s.eval(pts), Z[name + "/value"])
    assert np.array_equal(s.derivative(pts, Z[name + "/derivs"]), Z[name + "/deriv"])


def test_multithreaded_matches_single_thread():
    meta = [m for m in INDEX if m["name"] == "cube_3d_o3_20"][0]
    s1 = _spline(meta)
    s4 = oracle.Spline(meta["dim"], meta["order"], meta["periodic"], meta["sizes"], meta["lo"],
                       meta["hi"])
    s4.interpolate(Z[meta["name"] + "/values"].reshape(meta["sizes"]), nthreads=4)
    assert np.array_equal(s1.control_points(), s4.control_points())
    pts = np.random.default_rng(0).uniform(-1, 1, (5000, 3))
    assert np.array_equal(s1.eval(pts, 1), s1.eval(pts, 4))


REF_LIB = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                       "oracle", "_ref", "libintp_ref_cell.so")


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference not built on this host")
def test_live_reference_random_cases():
    """Fresh random cases against the live reference build, where it exists."""
    ref = C.CDLL(REF_LIB)
    Pv = C.c_void_p
    ref.ref_create.restype = Pv
    ref.ref_create.argtypes = [C.c_int, C.c_int, Pv, Pv, Pv, Pv, Pv, Pv]
    ref.ref_eval.argtypes = [Pv, Pv, C.c_int64, Pv, C.c_int]
    ref.ref_eval_deriv.argtypes = [Pv, Pv, C.c_int64, Pv, C.c_int, Pv, C.c_int]
    ref.ref_free.argtypes = [Pv]
    rng = np.random.default_rng(99)
    for _ in range(40):
        D = int(rng.integers(1, 4))
        O = int(rng.integers(0, 8))
        per = rng.integers(0, 2, D).astype(np.int32)
        sizes = rng.integers(max(O + 3, 4), 12, D).astype(np.int64)
        lo = rng.uniform(-1, 1, D)
        hi = lo + rng.uniform(0.5, 2, D)
        vals = rng.standard_normal(int(np.prod(sizes)))
        cptr = (Pv * D)()
        h = ref.ref_create(D, O, per.ctypes.data, sizes.ctypes.data, lo.ctypes.data,
                           hi.ctypes.data, cptr, vals.ctypes.data)
        s = oracle.Spline(D, O, per, sizes, lo, hi).interpolate(vals.reshape(sizes))
        pts = np.ascontiguousarray(rng.uniform(lo - 0.5, hi + 0.5, (100, D)))
        a = np.zeros(100)
        ref.ref_eval(h, pts.ctypes.data, 100, a.ctypes.data, 1)
        assert np.array_equal(a, s.eval(pts))
        ks = np.ascontiguousarray(rng.integers(0, O + 2, (2, D)), np.int32)
        da = np.zeros(200)
        ref.ref_eval_deriv(h, pts.ctypes.data, 100, ks.ctypes.data, 2, da.ctypes.data, 1)
        assert np.array_equal(da.reshape(100, 2), s.derivative(pts, ks))
        ref.ref_free(h)
