"""The MATLAB binding (bsplineinterpolation_gb300/matlab/): its MEX gateway
compiles against the C MEX API's declarations (CPU), and its core, given the
reference MEX function's MATLAB-layout arguments (column-major mesh and
coordinates, one range row / periodic flag / derivative order per MATLAB
dimension, reversed against the C++ axes as matlab/bspline.cpp does),
reproduces the reference's golden vectors on the GPU."""
import ctypes as C
import os
import shutil
import subprocess

import numpy as np
import pytest

from tests.golden_cases import expected, full_f, reference_cases, rel_err

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MATLAB_DIR = os.path.join(REPO, "bsplineinterpolation_gb300", "matlab")
LIBDIR = os.path.join(REPO, "bsplineinterpolation_gb300")
BUILD = os.path.join(REPO, "tests", "cpp", "_build")
SHIM = os.path.join(BUILD, "libmex_core_shim.so")
INC = ["-I" + os.path.join(REPO, "include"), "-I" + MATLAB_DIR]


def _gxx():
    if shutil.which("g++") is None:
        pytest.skip("no host compiler")
    return "g++"


def test_mex_gateway_compiles_against_the_mex_api():
    subprocess.check_call([_gxx(), "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only"] + INC +
                          ["-I" + os.path.join(REPO, "tests", "cpp", "fake_mex"),
                           os.path.join(MATLAB_DIR, "bspline_gpu.cpp")])


def _shim():
    from bsplineinterpolation_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    os.makedirs(BUILD, exist_ok=True)
    subprocess.check_call([_gxx(), "-std=c++17", "-O2", "-Wall", "-Wextra", "-fPIC", "-shared"] + INC +
                          [os.path.join(REPO, "tests", "cpp", "mex_core_shim.cpp"), "-o", SHIM,
                           "-L" + LIBDIR, "-lintp_gb300", "-Wl,-rpath," + LIBDIR])
    return SHIM


def test_mex_core_builds():
    assert os.path.exists(_shim())


def _matlab_call(lib, c):
    """The case in the reference MEX's conventions: MATLAB dimension j is
    C++ axis D-1-j."""
    D = c["dim"]
    sizes = list(c["sizes"])
    mesh = np.asarray(c["values"], np.float64)  # row-major C mesh = column-major reversed-dims MATLAB array
    dims = np.asarray(sizes[::-1], np.uint64)
    per = np.asarray([int(p) for p in c["periodic"][::-1]], np.uint8)
    rng = np.asarray(c["ranges"][::-1], np.float64)             # dim x 2
    rng_cm = np.asfortranarray(rng).ravel(order="F")             # column-major
    pts = np.asarray(c["points"], np.float64).reshape(-1, D)
    coords_cm = np.asfortranarray(pts[:, ::-1]).ravel(order="F")  # npts x dim, column-major
    ders = (c.get("derivs") or [[0] * D])[0]
    der = np.asarray(ders[::-1], np.uint64)
    out = np.zeros(pts.shape[0], np.float64)
    err = C.create_string_buffer(512)
    p = lambda a: a.ctypes.data_as(C.c_void_p)
    rc = lib.mex_core_eval(C.c_uint64(c["order"]), D, p(per), p(rng_cm), p(mesh), p(dims), p(coords_cm),
                           C.c_uint64(pts.shape[0]), p(der), p(out), err, 512)
    assert rc == 0, err.value
    return out


@pytest.mark.gpu
def test_mex_core_golden_vectors():
    lib = C.CDLL(_shim())
    lib.mex_core_eval.restype = C.c_int
    cases = reference_cases()
    f13 = full_f(cases)
    n = 0
    for c in cases:
        if c["kind"] != "interp" or c.get("coords"):
            continue  # the MEX function takes uniform axes only
        got = _matlab_call(lib, c)
        want = expected(c, f13)
        # the reference's own checks (as the C++ drop-in's test applies them)
        if c["name"].endswith(("extrapolation", "wrap")):
            assert np.max(np.abs(got - want)) < c["tol"], c["cite"]
        else:
            assert rel_err(got, want) < c["tol"], c["cite"]
        n += 1
    assert n >= 10
