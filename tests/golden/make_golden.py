"""Generate the golden fixtures under tests/golden/.

Run where the reference source tree is available (it is read, never copied):

    python tests/golden/make_golden.py --reference <reference root>

(or with INTP_REFERENCE_ROOT=<reference root> in the environment).

It writes two files:

* ``reference_tests.json`` -- the known-answer vectors of the reference's own
  tests (Mathematica values in test/src/interpolation-test.cpp and
  test/src/bspline-test.cpp), extracted from the test sources as text, with the
  inputs they are evaluated on and the tolerance those tests use.
* ``ref_outputs.npz`` -- outputs of the reference library itself (its headers
  compiled through oracle/build_ref.sh) on small seeded cases: control points,
  knot spans, values and derivatives. GPU tests compare against these without
  needing the reference tree.
"""
import argparse
import ctypes as C
import json
import os
import re
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def _initializer(src, name):
    """Brace-balanced initializer text following the declaration of `name`."""
    m = re.search(r"\b" + re.escape(name) + r"\s*(=\s*)?\{", src)
    if not m:
        raise KeyError(name)
    i = m.end() - 1
    depth = 0
    for j in range(i, len(src)):
        if src[j] == "{":
            depth += 1
        elif src[j] == "}":
            depth -= 1
            if depth == 0:
                return src[i: j + 1], src[: m.start()].count("\n") + 1, src[: j].count("\n") + 1
    raise ValueError(name)


_NUM = re.compile(r"^[\s\d\.\+\-\*/eE\(\)]+$")


def _values(text):
    body = text.replace("{", " ").replace("}", " ")
    out = []
    for item in body.split(","):
        item = item.strip()
        if not item:
            continue
        item = re.sub(r"(?<=[\d\.])[fF]\b", "", item)
        if not _NUM.match(item):
            raise ValueError("not numeric: %r" % item)
        out.append(float(eval(item, {"__builtins__": {}}, {})))
    return out


def extract(path, name):
    src = open(path).read()
    text, l0, l1 = _initializer(src, name)
    return _values(text), "%s:%d-%d" % (os.path.relpath(path, REF_ROOT), l0, l1)


def reference_tests():
    it = os.path.join(REF_ROOT, "test/src/interpolation-test.cpp")
    bt = os.path.join(REF_ROOT, "test/src/bspline-test.cpp")
    cases = []
    cite = {}

    def get(path, name):
        v, c = extract(path, name)
        cite[name] = c
        return v

    f, _ = extract(it, "f"), None
    f = f[0]
    cite["f"] = extract(it, "f")[1]
    c1h = get(it, "coords_1d_half")
    c1 = get(it, "coords_1d")
    f2 = get(it, "f2")
    c2 = get(it, "coords_2d")
    f3 = get(it, "f3")
    c3 = get(it, "coords_3d")
    xnu = get(it, "input_coords_1d")
    ynu2 = get(it, "nonuniform_coord_for_2d")
    tol = 1e-14

    def interp(name, dim, order, periodic, sizes, values, points, expected,
               ranges=None, coords=None, derivs=None, tol=tol, src=None):
        cases.append(dict(name=name, kind="interp", dim=dim, order=order,
                          periodic=periodic, sizes=sizes, values=values,
                          ranges=ranges, coords=coords, points=points,
                          derivs=derivs, expected=expected, tol=tol,
                          cite=src))

    # 1D uniform (interpolation-test.cpp:24-29)
    interp("1d_cubic", 1, 3, [False], [13], f, c1h, get(it, "vals_1d"),
           ranges=[[0.0, 6.0]], src=cite["vals_1d"])
    interp("1d_linear", 1, 1, [False], [13], f, c1, None, ranges=[[0.0, 12.0]],
           src="test/src/interpolation-test.cpp:44-54 (computed in-test)")
    interp("1d_segment", 1, 0, [False], [13], f, c1, None, ranges=[[0.0, 12.0]],
           src="test/src/interpolation-test.cpp:44-54 (computed in-test)")
    src = open(it).read()
    ext = [(float(a), float(b)) for a, b in
           re.findall(r"interp1\((-?[\d\.]+)\) - \((-?[\d\.e-]+)\)", src)]
    interp("1d_cubic_extrapolation", 1, 3, [False], [13], f, [e[0] for e in ext],
           [e[1] for e in ext], ranges=[[0.0, 6.0]],
           src="test/src/interpolation-test.cpp:92-101")
    interp("2d_cubic", 2, 3, [False, False], [5, 5], f2, c2, get(it, "vals_2d"),
           ranges=[[0.0, 4.0], [0.0, 4.0]], src=cite["vals_2d"])
    interp("3d_cubic", 3, 3, [False] * 3, [5, 6, 7], f3, c3, get(it, "vals_3d"),
           ranges=[[0.0, 4.0], [0.0, 5.0], [0.0, 6.0]], src=cite["vals_3d"])
    fp = f[:12]
    interp("1d_periodic_quartic", 1, 4, [True], [12], fp, c1,
           get(it, "vals_1d_periodic"), ranges=[[0.0, 12.0]],
           src=cite["vals_1d_periodic"])
    interp("1d_periodic_linear", 1, 1, [True], [12], fp, c1, None,
           ranges=[[0.0, 12.0]], src="test/src/interpolation-test.cpp:334-343 (computed in-test)")
    interp("1d_periodic_segment", 1, 0, [True], [12], fp, c1, None,
           ranges=[[0.0, 12.0]], src="test/src/interpolation-test.cpp:334-343 (computed in-test)")
    vp = get(it, "vals_1d_periodic")
    interp("1d_periodic_wrap", 1, 4, [True], [12], fp,
           [c1[0] - 12.0, c1[0] + 12.0], [vp[0], vp[0]], ranges=[[0.0, 12.0]],
           src="test/src/interpolation-test.cpp:379-384")
    f2py = [f2[i * 5 + j] for i in range(5) for j in range(4)]
    interp("2d_y_periodic", 2, 3, [False, True], [5, 4], f2py, c2,
           get(it, "vals_2d_periodic"), ranges=[[0.0, 4.0], [0.0, 4.0]],
           src=cite["vals_2d_periodic"])
    interp("1d_derivative", 1, 3, [False], [13], f, c1h,
           get(it, "vals_1d_derivative_1"), ranges=[[0.0, 6.0]], derivs=[[1]],
           src=cite["vals_1d_derivative_1"])
    interp("1d_periodic_derivative", 1, 4, [True], [12], fp, c1,
           get(it, "vals_1d_derivative_periodic"), ranges=[[0.0, 12.0]],
           derivs=[[1]], src=cite["vals_1d_derivative_periodic"])
    interp("2d_derivative_x2_y1", 2, 3, [False, False], [5, 5], f2, c2,
           get(it, "vals_2d_derivative_x2_y1"), ranges=[[0.0, 4.0], [0.0, 4.0]],
           derivs=[[2, 1]], src=cite["vals_2d_derivative_x2_y1"])
    interp("3d_derivative_x1_y0_z3", 3, 3, [False] * 3, [5, 6, 7], f3, c3,
           get(it, "vals_3d_derivative_x1_y0_z3"),
           ranges=[[0.0, 4.0], [0.0, 5.0], [0.0, 6.0]], derivs=[[1, 0, 3]],
           src=cite["vals_3d_derivative_x1_y0_z3"])
    interp("1d_nonuniform_cubic", 1, 3, [False], [13], f, c1,
           get(it, "vals_1d_nonuniform"), coords=[xnu],
           src=cite["vals_1d_nonuniform"])
    interp("1d_nonuniform_linear", 1, 1, [False], [13], f, c1, None, coords=[xnu],
           src="test/src/interpolation-test.cpp:540-551 (computed in-test)")
    interp("1d_nonuniform_periodic_quartic", 1, 4, [True], [12], fp, c1,
           get(it, "vals_1d_nonuniform_periodic"), coords=[xnu],
           src=cite["vals_1d_nonuniform_periodic"])
    interp("1d_nonuniform_periodic_linear", 1, 1, [True], [12], fp, c1, None,
           coords=[xnu], src="test/src/interpolation-test.cpp:595-606 (computed in-test)")
    f2px = f2[:20]
    interp("2d_x_periodic_y_nonuniform", 2, 3, [True, False], [4, 5], f2px, c2,
           get(it, "vals_2d_X_periodic_Y_nonuniform"),
           ranges=[[0.0, 4.0], None], coords=[None, ynu2],
           src=cite["vals_2d_X_periodic_Y_nonuniform"])
    cases.append(dict(name="2d_at_out_of_range", kind="domain_error", dim=2, order=3,
                      periodic=[False, False], sizes=[5, 5], values=f2,
                      ranges=[[0.0, 4.0], [0.0, 4.0]], coords=None,
                      points=[-1.0, 1.0], cite="test/src/interpolation-test.cpp:159-164"))

    # bspline-test.cpp: splines given by knots and control points, tol 1e-15
    knots = get(bt, "knots")
    cp = get(bt, "cp")
    cp2 = get(bt, "cp2")
    cp3 = get(bt, "cp3")
    knots2 = get(bt, "knots2")
    bc1 = extract(bt, "coords_1d")[0]
    bc2 = extract(bt, "coords_2d")[0]
    bc3 = extract(bt, "coords_3d")[0]
    btol = 1e-15

    def spline(name, dim, periodic, ncp, kn, ctrl, points, expected, derivs=None, src=None):
        cases.append(dict(name=name, kind="bspline", dim=dim, order=3,
                          periodic=periodic, ncp=ncp, knots=kn, ctrl=ctrl,
                          points=points, derivs=derivs, expected=expected,
                          tol=btol, cite=src))

    bv1, c = extract(bt, "vals_1d")
    spline("bspline_1d", 1, [False], [5], [knots], cp, bc1, bv1, src=c)
    bv2, c = extract(bt, "vals_2d")
    spline("bspline_2d", 2, [False, False], [5, 5], [knots, knots], cp2, bc2, bv2, src=c)
    bv3, c = extract(bt, "vals_3d")
    spline("bspline_3d", 3, [False] * 3, [5, 5, 5], [knots] * 3, cp3, bc3, bv3, src=c)
    bvp, c = extract(bt, "vals_2d_periodic")
    spline("bspline_2d_periodic", 2, [False, True], [5, 5], [knots, knots2], cp2, bc2, bvp, src=c)
    spline("bspline_1d_derivative_0", 1, [False], [5], [knots], cp, bc1, bv1, derivs=[[0]],
           src="test/src/bspline-test.cpp:255-264 (derivative 0 against vals_1d)")
    v, c = extract(bt, "vals_1d_derivative_1")
    spline("bspline_1d_derivative_1", 1, [False], [5], [knots], cp, bc1, v, derivs=[[1]], src=c)
    v, c = extract(bt, "vals_1d_derivative_2")
    spline("bspline_1d_derivative_2", 1, [False], [5], [knots], cp, bc1, v, derivs=[[2]], src=c)
    v, c = extract(bt, "vals_2d_derivative_x2_y0")
    spline("bspline_2d_derivative_x2_y0", 2, [False, False], [5, 5], [knots, knots], cp2, bc2,
           v, derivs=[[2, 0]], src=c)
    v, c = extract(bt, "vals_2d_derivative_x1_y1")
    spline("bspline_2d_derivative_x1_y1", 2, [False, False], [5, 5], [knots, knots], cp2, bc2,
           v, derivs=[[1, 1]], src=c)
    v, c = extract(bt, "vals_2d_periodic_derivative_x1_y1")
    spline("bspline_2d_periodic_derivative_x1_y1", 2, [False, True], [5, 5], [knots, knots2],
           cp2, bc2, v, derivs=[[1, 1]], src=c)
    return cases


# ---------------------------------------------------------------------------
# reference outputs on seeded cases
# ---------------------------------------------------------------------------
def _ref_lib():
    path = os.path.join(REPO, "oracle", "_ref", "libintp_ref_cell.so")
    pathp = os.path.join(REPO, "oracle", "_ref", "libintp_ref_plain.so")
    if not os.path.exists(path) or not os.path.exists(pathp):
        subprocess.check_call(["sh", os.path.join(REPO, "oracle", "build_ref.sh")],
                              env=dict(os.environ, INTP_REFERENCE_ROOT=REF_ROOT))
    libs = []
    for p in (path, pathp):
        lib = C.CDLL(p)
        P = C.c_void_p
        lib.ref_create.restype = P
        lib.ref_create.argtypes = [C.c_int, C.c_int, P, P, P, P, P, P]
        lib.ref_eval.argtypes = [P, P, C.c_int64, P, C.c_int]
        lib.ref_eval_deriv.argtypes = [P, P, C.c_int64, P, C.c_int, P, C.c_int]
        lib.ref_num_ctrl.restype = C.c_int64
        lib.ref_num_ctrl.argtypes = [P]
        lib.ref_ctrl.argtypes = [P, P]
        lib.ref_locate.argtypes = [P, P, C.c_int64, P, P]
        lib.ref_num_knots.restype = C.c_int64
        lib.ref_num_knots.argtypes = [P, C.c_int]
        lib.ref_knots.argtypes = [P, C.c_int, P]
        lib.ref_range.argtypes = [P, C.c_int, P, P]
        lib.ref_free.argtypes = [P]
        lib.ref_last_error.restype = C.c_char_p
        libs.append(lib)
    return libs


def seeded_cases():
    """Small seeded cases covering D=1..3, orders 0..7, periodic/non-periodic,
    uniform/non-uniform axes, and the BASELINE workload shapes at reduced size."""
    rng = np.random.default_rng(20261203)
    cases = []
    # the plain-method workload: 2D, order 3, 64x64 on [0,1]x[0,2],
    # z = sin(3x)cos(2y) + N(0, 0.01^2), 1e4 uniform points in the domain
    x = np.linspace(0, 1, 64)
    y = np.linspace(0, 2, 64)
    z = np.sin(3 * x)[:, None] * np.cos(2 * y)[None, :] + rng.normal(0, 0.01, (64, 64))
    cases.append(dict(name="plain_2d_o3_64x64", dim=2, order=3, periodic=[0, 0],
                      sizes=[64, 64], lo=[0.0, 0.0], hi=[1.0, 2.0], coords=[None, None],
                      values=z.ravel(), npts=3000, domain_only=True,
                      derivs=[[0, 0], [1, 0], [0, 1], [2, 0], [1, 1], [0, 2]]))
    # periodic high order at reduced size: 2D order 7, 48x40
    kx = rng.integers(1, 6, 16)
    ky = rng.integers(1, 6, 16)
    ph = rng.uniform(0, 2 * np.pi, 16)
    gx = np.arange(48) * (2 * np.pi / 48)
    gy = np.arange(40) * (2 * np.pi / 40)
    v = sum(np.sin(kx[i] * gx[:, None] + ky[i] * gy[None, :] + ph[i]) for i in range(16))
    cases.append(dict(name="periodic_2d_o7_48x40", dim=2, order=7, periodic=[1, 1],
                      sizes=[48, 40], lo=[0.0, 0.0], hi=[2 * np.pi, 2 * np.pi],
                      coords=[None, None], values=v.ravel(), npts=2000, domain_only=False,
                      derivs=[[1, 0], [0, 1], [2, 0], [1, 1], [0, 2]]))
    # 3D cubic non-periodic at reduced size (the 256^3 workload's shape)
    n = 20
    g = np.linspace(-1, 1, n)
    X, Y, Z = np.meshgrid(g, g, g, indexing="ij")
    f = np.exp(-(X ** 2 + Y ** 2 + Z ** 2)) * np.cos(4 * X) + rng.normal(0, 1e-3, X.shape)
    cases.append(dict(name="cube_3d_o3_20", dim=3, order=3, periodic=[0, 0, 0],
                      sizes=[n, n, n], lo=[-1.0] * 3, hi=[1.0] * 3, coords=[None] * 3,
                      values=f.ravel(), npts=2000, domain_only=False,
                      derivs=[[0, 0, 0], [1, 0, 0], [0, 2, 1], [3, 3, 3], [4, 0, 0]]))
    # sweep of orders / periodicity / non-uniform axes
    for k in range(40):
        D = int(rng.integers(1, 4))
        O = int(rng.integers(0, 8))
        per = [int(v) for v in rng.integers(0, 2, D)]
        sizes = [int(s) for s in rng.integers(max(O + 3, 4), 17, D)]
        lo = rng.uniform(-2, 1, D)
        hi = lo + rng.uniform(0.5, 3, D)
        coords = [None] * D
        if D <= 2:
            for d in range(D):
                if rng.random() < 0.4 and not (O == 0 and not per[d]):
                    m = sizes[d] + per[d]
                    c = np.sort(rng.uniform(lo[d], hi[d], m))
                    c[0], c[-1] = lo[d], hi[d]
                    coords[d] = c
        derivs = [[int(v) for v in rng.integers(0, O + 2, D)] for _ in range(3)]
        cases.append(dict(name="sweep_%02d_d%d_o%d" % (k, D, O), dim=D, order=O,
                          periodic=per, sizes=sizes, lo=list(lo), hi=list(hi),
                          coords=coords, values=rng.standard_normal(int(np.prod(sizes))),
                          npts=300, domain_only=False, derivs=derivs))
    return cases


def ref_outputs(path):
    lib, libp = _ref_lib()
    P = C.c_void_p
    rng = np.random.default_rng(7)
    arrays = {}
    index = []
    for case in seeded_cases():
        D = case["dim"]
        per = np.array(case["periodic"], np.int32)
        sizes = np.array(case["sizes"], np.int64)
        lo = np.array(case["lo"], np.float64)
        hi = np.array(case["hi"], np.float64)
        vals = np.ascontiguousarray(case["values"], np.float64)
        coords = [None if c is None else np.ascontiguousarray(c, np.float64) for c in case["coords"]]
        cptr = (P * D)(*[None if c is None else c.ctypes.data for c in coords])
        h = lib.ref_create(D, case["order"], per.ctypes.data, sizes.ctypes.data,
                           lo.ctypes.data, hi.ctypes.data, cptr, vals.ctypes.data)
        hp = libp.ref_create(D, case["order"], per.ctypes.data, sizes.ctypes.data,
                             lo.ctypes.data, hi.ctypes.data, cptr, vals.ctypes.data)
        if not h or not hp:
            raise RuntimeError(lib.ref_last_error())
        # domain per axis from the reference's own range()
        rlo = np.zeros(D)
        rhi = np.zeros(D)
        for d in range(D):
            a, b = C.c_double(), C.c_double()
            lib.ref_range(h, d, C.byref(a), C.byref(b))
            rlo[d], rhi[d] = a.value, b.value
        npts = case["npts"]
        span = rhi - rlo
        if case["domain_only"]:
            pts = rng.uniform(rlo, rhi, (npts, D))
        else:
            # include out-of-range points: extrapolation and periodic wrap
            pts = rng.uniform(rlo - 0.25 * span, rhi + 0.25 * span, (npts, D))
            # exact knot hits and range ends
            kn = [np.zeros(lib.ref_num_knots(h, d)) for d in range(D)]
            for d in range(D):
                lib.ref_knots(h, d, kn[d].ctypes.data)
            for r in range(min(npts // 4, 64)):
                for d in range(D):
                    pts[r, d] = kn[d][rng.integers(0, len(kn[d]))]
            pts[-1] = rlo
            pts[-2] = rhi
        pts = np.ascontiguousarray(pts)
        val = np.zeros(npts)
        lib.ref_eval(h, pts.ctypes.data, npts, val.ctypes.data, 1)
        ks = np.ascontiguousarray(case["derivs"], np.int32)
        K = ks.shape[0]
        der = np.zeros(npts * K)
        lib.ref_eval_deriv(h, pts.ctypes.data, npts, ks.ctypes.data, K, der.ctypes.data, 1)
        cells = np.zeros((npts, D), np.int64)
        wrapped = np.zeros((npts, D))
        lib.ref_locate(h, pts.ctypes.data, npts, cells.ctypes.data, wrapped.ctypes.data)
        ctrl = np.zeros(libp.ref_num_ctrl(hp))
        libp.ref_ctrl(hp, ctrl.ctypes.data)
        name = case["name"]
        arrays[name + "/values"] = vals
        arrays[name + "/points"] = pts
        arrays[name + "/value"] = val
        arrays[name + "/derivs"] = ks
        arrays[name + "/deriv"] = der.reshape(npts, K)
        arrays[name + "/cells"] = cells
        arrays[name + "/wrapped"] = wrapped
        arrays[name + "/ctrl"] = ctrl
        for d in range(D):
            kn = np.zeros(lib.ref_num_knots(h, d))
            lib.ref_knots(h, d, kn.ctypes.data)
            arrays[name + "/knots%d" % d] = kn
            if coords[d] is not None:
                arrays[name + "/coords%d" % d] = coords[d]
        arrays[name + "/range"] = np.stack([rlo, rhi], axis=1)
        index.append(dict(name=name, dim=D, order=case["order"],
                          periodic=case["periodic"], sizes=case["sizes"],
                          lo=[float(v) for v in lo], hi=[float(v) for v in hi],
                          nonuniform=[c is not None for c in coords]))
        lib.ref_free(h)
        libp.ref_free(hp)
    arrays["index"] = np.frombuffer(json.dumps(index).encode(), np.uint8)
    np.savez_compressed(path, **arrays)


def main():
    global REF_ROOT
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("INTP_REFERENCE_ROOT"),
                    help="root of the reference source tree (or INTP_REFERENCE_ROOT)")
    args = ap.parse_args()
    if not args.reference:
        ap.error("the reference root is required (--reference or INTP_REFERENCE_ROOT)")
    REF_ROOT = os.path.abspath(args.reference)
    cases = reference_tests()
    with open(os.path.join(HERE, "reference_tests.json"), "w") as fh:
        json.dump(dict(generator="tests/golden/make_golden.py",
                       note="known-answer vectors of the reference's own tests",
                       cases=cases), fh, indent=1)
    ref_outputs(os.path.join(HERE, "ref_outputs.npz"))
    print("wrote", os.path.join(HERE, "reference_tests.json"), "and ref_outputs.npz")


REF_ROOT = None  # set by main()

if __name__ == "__main__":
    sys.exit(main())
