"""The header-only C++ drop-in (include/intp/) used like the reference:
compiled here against the reference-shaped API (CPU), and run on a GPU
against the golden vectors of test/src/interpolation-test.cpp."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests.golden_cases import expected, full_f, reference_cases, rel_err

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(REPO, "tests", "cpp", "dropin_test.cpp")
BIN = os.path.join(REPO, "tests", "cpp", "_build", "dropin_test")
LIBDIR = os.path.join(REPO, "bsplineinterpolation_gb300")

CASES = [c for c in reference_cases() if c["kind"] == "interp"]
F13 = full_f(reference_cases())


def _compile():
    if shutil.which("g++") is None:
        pytest.skip("no host compiler")
    from bsplineinterpolation_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    os.makedirs(os.path.dirname(BIN), exist_ok=True)
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-I" + os.path.join(REPO, "include"),
                           SRC, "-o", BIN, "-L" + LIBDIR, "-lintp_gb300", "-Wl,-rpath," + LIBDIR])
    return BIN


def test_dropin_compiles():
    assert os.path.exists(_compile())


def _encode(c):
    D = c["dim"]
    parts = [c["name"], str(D), str(c["order"])]
    parts += [str(int(p)) for p in c["periodic"]] + [str(s) for s in c["sizes"]]
    coords = c.get("coords") or [None] * D
    ranges = c.get("ranges") or [None] * D
    for d in range(D):
        if coords[d] is None:
            parts += ["U", float(ranges[d][0]).hex(), float(ranges[d][1]).hex()]
        else:
            parts += ["N", str(len(coords[d]))] + [float(v).hex() for v in coords[d]]
    parts += [str(len(c["values"]))] + [float(v).hex() for v in c["values"]]
    pts = np.asarray(c["points"], np.float64).reshape(-1, D)
    parts += [str(pts.shape[0])] + [float(v).hex() for v in pts.ravel()]
    ks = c.get("derivs") or []
    parts += [str(len(ks))] + [str(int(v)) for row in ks for v in row]
    return " ".join(parts)


@pytest.mark.gpu
def test_dropin_golden_vectors():
    exe = _compile()
    inp = "\n".join(_encode(c) for c in CASES) + "\n"
    r = subprocess.run([exe], input=inp, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    out = {line.split()[0]: line.split()[1:] for line in r.stdout.splitlines()}
    for c in CASES:
        row = out[c["name"]]
        assert row[0] not in ("error", "unsupported"), (c["name"], row)
        n = int(row[0])
        vals = np.array([float.fromhex(v) for v in row[1:]])
        single, batch = vals[:n], vals[n:]
        want = expected(c, F13)
        assert np.array_equal(single, batch), c["name"]
        if c["name"].endswith(("extrapolation", "wrap")):
            assert np.max(np.abs(single - want)) < c["tol"], c["cite"]
        else:
            assert rel_err(single, want) < c["tol"], c["cite"]


@pytest.mark.gpu
def test_dropin_reference_shaped_usage():
    exe = _compile()
    r = subprocess.run([exe, "extras"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "extras 0" in r.stdout, r.stdout + r.stderr
