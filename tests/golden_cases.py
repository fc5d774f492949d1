"""Loading of the golden fixtures and the in-test expectations that the
reference's tests compute themselves (test/src/interpolation-test.cpp)."""
import json
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def reference_cases():
    with open(os.path.join(GOLDEN, "reference_tests.json")) as fh:
        return json.load(fh)["cases"]


def ref_outputs():
    z = np.load(os.path.join(GOLDEN, "ref_outputs.npz"))
    index = json.loads(bytes(z["index"]).decode())
    return z, index


def rel_err(got, want):
    """RMS relative error of test/src/include/rel_err.hpp:11-49."""
    got = np.asarray(got, np.float64).ravel()
    want = np.asarray(want, np.float64).ravel()
    return math.sqrt(float(np.sum((got - want) ** 2)) / float(np.sum(want ** 2)))


def _round_half_away(x):
    return math.floor(x + 0.5) if x >= 0 else -math.floor(-x + 0.5)


def expected(case, full_f=None):
    """Expected values; computes the in-test ones (segment / linear) exactly as
    test/src/interpolation-test.cpp:44-54, :334-343, :540-551, :595-606 do."""
    if case.get("expected") is not None:
        return np.asarray(case["expected"], np.float64)
    name = case["name"]
    f = full_f
    pts = case["points"]
    out = []
    for x in pts:
        if name in ("1d_linear",):
            i = int(math.floor(x))
            out.append(f[i] + (f[i + 1] - f[i]) * (x - i))
        elif name in ("1d_segment", "1d_periodic_segment"):
            out.append(f[_round_half_away(x)])
        elif name == "1d_periodic_linear":
            i = int(math.floor(x))
            out.append(f[i] + (f[(i + 1) % (len(f) - 1)] - f[i]) * (x - i))
        elif name in ("1d_nonuniform_linear", "1d_nonuniform_periodic_linear"):
            c = case["coords"][0]
            i = int(np.searchsorted(c, x, side="left"))
            nxt = f[i] if name == "1d_nonuniform_linear" else f[i % (len(f) - 1)]
            out.append(f[i - 1] + (nxt - f[i - 1]) * (x - c[i - 1]) / (c[i] - c[i - 1]))
        else:
            raise KeyError(name)
    return np.asarray(out)


def full_f(cases):
    for c in cases:
        if c["name"] == "1d_cubic":
            return c["values"]
    raise KeyError("1d_cubic")
