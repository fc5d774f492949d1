"""Batched tables (intp_batch_*): many tables of uneven size, order,
periodicity and dimension built and evaluated together.

A batched table must give what the same table gives alone: the control
points of intp_table_interpolate bit for bit (the line solves run the same
substitution code), the direct kernel's outputs (the same per-point code),
and -- through those -- the reference's outputs at the single-table
tolerances: 1e-12 in the FP64 form, 1e-6 * max(1, kappa) in the mixed form.
"""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bsplineinterpolation_gb300 as bi
from oracle import oracle
from tests.golden_cases import ref_outputs
from tests.gpu_util import norm_rel_err

pytestmark = pytest.mark.gpu

Z, INDEX = ref_outputs()
BATCHABLE = [m for m in INDEX if m["dim"] <= 3]


def _ranges(meta):
    name = meta["name"]
    return [Z[name + "/coords%d" % d] if meta["nonuniform"][d] else (meta["lo"][d], meta["hi"][d])
            for d in range(meta["dim"])]


def _golden_batch(precision):
    specs = [(m["order"], m["periodic"], m["sizes"], _ranges(m)) for m in BATCHABLE]
    b = bi.TableBatch(specs, precision=precision)
    b.build([Z[m["name"] + "/values"] for m in BATCHABLE])
    return b


def _batch_points(metas, key="/points"):
    pts = [Z[m["name"] + key] for m in metas]
    offsets = np.concatenate([[0], np.cumsum([p.shape[0] for p in pts])]).astype(np.int64)
    flat = torch.tensor(np.concatenate([p.ravel() for p in pts]), device="cuda")
    return pts, offsets, flat


def _derivs4(rows):
    rows = np.asarray(rows, np.int32)
    out = np.zeros((rows.shape[0], 4), np.int32)
    out[:, :rows.shape[1]] = rows
    return out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_control_points_equal_single_tables(precision):
    b = _golden_batch(precision)
    for i, m in enumerate(BATCHABLE):
        mesh = Z[m["name"] + "/values"].reshape(m["sizes"])
        f = bi.InterpolationFunction(m["order"], m["periodic"], torch.tensor(mesh, device="cuda"),
                                     *_ranges(m), precision=precision)
        assert np.array_equal(b.control_points(i), f.control_points()), m["name"]
        if precision == "fp64":
            assert norm_rel_err(b.control_points(i).ravel(), Z[m["name"] + "/ctrl"]) < 1e-12, m["name"]


def test_batch_fp64_values_match_reference():
    b = _golden_batch("fp64")
    pts, offsets, flat = _batch_points(BATCHABLE)
    val = b.evaluate(flat, offsets).cpu().numpy()[:, 0]
    for i, m in enumerate(BATCHABLE):
        got = val[offsets[i]:offsets[i + 1]]
        assert norm_rel_err(got, Z[m["name"] + "/value"]) < 1e-12, m["name"]


def test_batch_fp64_derivatives_match_reference():
    """Derivative rows differ per table in the golden set, so each dimension
    class is evaluated with a shared request and compared with the oracle."""
    b = _golden_batch("fp64")
    pts, offsets, flat = _batch_points(BATCHABLE)
    req = [[1, 0, 0], [0, 1, 0], [2, 0, 1]]
    got = b.evaluate(flat, offsets, derivs=_derivs4(req)).cpu().numpy()
    for i, m in enumerate(BATCHABLE):
        D = m["dim"]
        s = oracle.Spline(D, m["order"], m["periodic"], m["sizes"], m["lo"], m["hi"],
                          coords=[Z[m["name"] + "/coords%d" % d] if m["nonuniform"][d] else None
                                  for d in range(D)])
        s.interpolate(Z[m["name"] + "/values"])
        want = s.derivative(pts[i], np.asarray(req)[:, :D])
        assert norm_rel_err(got[offsets[i]:offsets[i + 1]], want) < 1e-12, m["name"]


def test_batch_mixed_equals_direct_kernel():
    """Mixed batch outputs against each table evaluated alone by the direct
    kernel (the batched kernel runs the same per-point code)."""
    b = _golden_batch("mixed")
    pts, offsets, flat = _batch_points(BATCHABLE)
    req = [[0, 0, 0], [1, 0, 0]]
    got = b.evaluate(flat, offsets, derivs=_derivs4(req)).double().cpu().numpy()
    old = os.environ.get("INTP_GB300_EVAL")
    os.environ["INTP_GB300_EVAL"] = "direct"
    try:
        for i, m in enumerate(BATCHABLE):
            D = m["dim"]
            mesh = Z[m["name"] + "/values"].reshape(m["sizes"])
            f = bi.InterpolationFunction(m["order"], m["periodic"], torch.tensor(mesh, device="cuda"),
                                         *_ranges(m), precision="mixed")
            want = f.evaluate(torch.tensor(pts[i], device="cuda"),
                              derivs=np.asarray(req)[:, :D]).double().cpu().numpy()
            g = got[offsets[i]:offsets[i + 1]]
            scale = np.maximum(np.max(np.abs(want), axis=0), 1e-300)
            assert np.all(np.abs(g - want) <= 1e-6 * scale), m["name"]
    finally:
        if old is None:
            os.environ.pop("INTP_GB300_EVAL", None)
        else:
            os.environ["INTP_GB300_EVAL"] = old


def _fourier_1d(rng, n, periodic):
    L = n if periodic else n - 1
    x = np.arange(n, dtype=np.float64)
    f = np.zeros(n)
    for k in range(1, 9):
        f += rng.normal(0.0, 1.0 / k) * np.cos(2 * np.pi * k * x / L + rng.uniform(0, 2 * np.pi))
    return f


def make_uneven_batch(ntables, seed, max_points=3000, max_1d=4096, max_2d=256):
    """Tables shaped like the batched workload: half 1D with N ~ U[16, max_1d],
    half 2D with sides ~ U[16, max_2d]; orders 3 or 5; 30% periodic (all axes);
    values are 8-mode random Fourier series (a product of two in 2D) with
    amplitudes ~ N(0, 1/k^2); each table gets uniform query points."""
    rng = np.random.default_rng(seed)
    specs, values, pts = [], [], []
    for i in range(ntables):
        order = int(rng.choice([3, 5]))
        periodic = bool(rng.random() < 0.3)
        if i % 2 == 0:
            n = int(rng.integers(16, max_1d + 1))
            dims = [n]
            v = _fourier_1d(rng, n, periodic)
        else:
            dims = [int(rng.integers(16, max_2d + 1)), int(rng.integers(16, max_2d + 1))]
            v = np.outer(_fourier_1d(rng, dims[0], periodic), _fourier_1d(rng, dims[1], periodic))
        ranges = [(0.0, float(d)) for d in dims]
        specs.append((order, [periodic] * len(dims), dims, ranges))
        values.append(v)
        npts = int(rng.integers(100, max_points + 1))
        pts.append(rng.uniform(0.0, [float(d) for d in dims], (npts, len(dims))))
    return specs, values, pts


def test_uneven_mixed_batch_against_oracle():
    specs, values, pts = make_uneven_batch(48, 20261206)
    b = bi.TableBatch(specs, precision="mixed")
    b.build(values)
    offsets = np.concatenate([[0], np.cumsum([p.shape[0] for p in pts])]).astype(np.int64)
    flat = torch.tensor(np.concatenate([p.ravel() for p in pts]), device="cuda")
    got = b.evaluate(flat, offsets).double().cpu().numpy()[:, 0]
    for i, (order, per, dims, ranges) in enumerate(specs):
        D = len(dims)
        s = oracle.Spline(D, order, per, dims, [r[0] for r in ranges], [r[1] for r in ranges])
        s.interpolate(values[i])
        want = s.eval(pts[i])
        kappa = float(np.max(np.abs(s.control_points())) / np.max(np.abs(values[i])))
        assert norm_rel_err(got[offsets[i]:offsets[i + 1]], want) < 1e-6 * max(1.0, kappa), (i, order, per, dims)


def test_batch_tables_without_points_and_empty_request():
    specs, values, pts = make_uneven_batch(6, 7)
    b = bi.TableBatch(specs, precision="mixed")
    b.build(torch.tensor(np.concatenate([v.ravel() for v in values]), device="cuda"))
    counts = [p.shape[0] for p in pts]
    counts[1] = 0
    counts[4] = 0
    offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    flat = torch.tensor(np.concatenate([p.ravel() for i, p in enumerate(pts) if counts[i]]), device="cuda")
    got = b.evaluate(flat, offsets).double().cpu().numpy()[:, 0]
    assert got.shape[0] == offsets[-1]
    empty = b.evaluate(torch.zeros(0, dtype=torch.float64, device="cuda"), np.zeros(7, np.int64))
    assert empty.shape[0] == 0


def test_batch_rejects_bad_requests():
    specs, values, _ = make_uneven_batch(4, 3)
    b = bi.TableBatch(specs, precision="mixed")
    with pytest.raises(bi.IntpError):  # evaluation before build
        b.evaluate(torch.zeros(2, dtype=torch.float64, device="cuda"), np.array([0, 1, 1, 1, 1]))
    b.build(values)
    with pytest.raises(bi.IntpError):  # decreasing offsets
        b.evaluate(torch.zeros(4, dtype=torch.float64, device="cuda"), np.array([0, 2, 1, 1, 1]))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_schedules_give_identical_control_points(precision):
    """The line solves' schedule (persistent work queue or one CTA per item,
    lines per item on the contiguous and the strided axes) never changes a
    line's arithmetic: every schedule, and the one intp_batch_autotune picks,
    gives the same control points bit for bit (and those of the tables built
    alone)."""
    b = _golden_batch(precision)
    want = [b.control_points(i) for i in range(len(BATCHABLE))]
    values = np.concatenate([Z[m["name"] + "/values"] for m in BATCHABLE])
    for persistent, crows, rows in ((False, 32, 32), (True, 1, 8), (True, 7, 1), (False, 16, 16)):
        b.set_schedule(persistent, crows, rows)
        assert b.schedule()["contig_rows"] == crows
        b.build(values)
        for i in range(len(BATCHABLE)):
            assert np.array_equal(b.control_points(i), want[i]), (persistent, crows, rows, BATCHABLE[i]["name"])
    chosen = b.autotune(values)
    assert chosen["build_ms"] > 0 and chosen["contig_rows"] in (16, 32)
    for i in range(len(BATCHABLE)):
        assert np.array_equal(b.control_points(i), want[i])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_vector_valued_tables_in_a_batch(precision):
    """Vector-valued tables (the reference's InterpolationFunction with a
    vector T, interpolation-test.cpp:672-703) mixed with scalar ones in one
    batch: each table's control points and outputs equal those of the same
    table built and evaluated alone, bit for bit, and every channel agrees
    with the oracle's scalar table of that channel."""
    rng = np.random.default_rng(41)
    tables = [  # (order, periodicity, dims, channels)
        (3, [False, False], [40, 36], 3),
        (5, [True], [300], 1),
        (3, [True, False], [33, 130], 2),
        (4, [False], [2000], 4),
        (5, [False, True, False], [12, 14, 16], 2),
        (3, [False, False], [20, 24], 1),
    ]
    specs, vals, per_table = [], [], []
    for order, per, dims, C in tables:
        v = rng.normal(size=list(dims) + ([C] if C > 1 else []))
        axes = np.meshgrid(*[np.linspace(0.0, 1.0, n) for n in dims], indexing="ij")
        smooth = np.cos(3.0 * axes[0]) * np.sin(2.0 * axes[-1] + 0.5)
        v = 1e-3 * v + (smooth[..., None] if C > 1 else smooth)
        ranges = [(0.0, 1.0)] * len(dims)
        specs.append((order, per, dims, ranges, C))
        vals.append(v.ravel())
        per_table.append(v)
    b = bi.TableBatch(specs, precision=precision)
    b.build(np.concatenate(vals))
    counts = [int(rng.integers(0, 3000)) for _ in tables]
    counts[1] = 0  # a table without points
    po = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    pts = [rng.uniform(0.0, 1.0, (n, len(t[2]))) for n, t in zip(counts, tables)]
    coords = torch.tensor(np.concatenate([p.ravel() for p in pts]), device="cuda")
    derivs = np.array([[0, 0, 0], [1, 0, 0]], np.int32)
    out = b.evaluate(coords, po, derivs=derivs, out_dtype="f64")
    views = b.output_views(out, po, K=2)
    for i, (order, per, dims, C) in enumerate(tables):
        ranges = [(0.0, 1.0)] * len(dims)
        f = bi.InterpolationFunction(order, per, per_table[i], *ranges, precision=precision, vector=C > 1)
        assert np.array_equal(b.control_points(i), f.control_points()), i
        if counts[i] == 0:
            assert views[i].shape[0] == 0
            continue
        want = f.evaluate(torch.tensor(pts[i], device="cuda"), derivs=derivs[:, :len(dims)],
                          out_dtype="f64").cpu().numpy()
        got = views[i].cpu().numpy()
        assert got.shape == want.shape, i
        assert np.array_equal(got, want), i
        tol = 1e-12 if precision == "fp64" else 1e-6
        for c in range(C):
            chan = per_table[i][..., c] if C > 1 else per_table[i]
            ref = oracle.Spline(len(dims), order, per, dims, [0.0] * len(dims), [1.0] * len(dims)).interpolate(chan)
            g = got[:, 0, c] if C > 1 else got[:, 0]
            assert norm_rel_err(g, ref.eval(pts[i])) < tol, (i, c)


@pytest.mark.parametrize("persistent", [False, True])
def test_captured_graph_equals_build_and_eval(persistent):
    """A CUDA graph of one build and one evaluation (intp_batch_graph_*):
    each replay gives what intp_batch_build + intp_batch_eval give on the
    buffers' contents at that time, bit for bit, also after the values and
    the coordinates are overwritten in place between replays."""
    specs, values, pts = make_uneven_batch(40, 20261211)
    b = bi.TableBatch(specs, precision="mixed")
    b.set_schedule(persistent, 32, 32)
    offsets = np.concatenate([[0], np.cumsum([p.shape[0] for p in pts])]).astype(np.int64)
    vals = torch.tensor(np.concatenate([v.ravel() for v in values]), device="cuda")
    coords = torch.tensor(np.concatenate([p.ravel() for p in pts]), device="cuda")
    derivs = np.array([[0, 0], [1, 0]], np.int32)
    g = b.graph(vals, coords, offsets, derivs=derivs)
    try:
        for step in range(3):
            if step > 0:
                vals.mul_(1.0 + 0.25 * step).add_(0.125)
                coords.mul_(0.999)
            out = g.launch()
            torch.cuda.synchronize()
            got = out.clone()
            b.build(vals)
            want = b.evaluate(coords, offsets, derivs=derivs)
            torch.cuda.synchronize()
            assert torch.equal(got.reshape(want.shape), want), step
        # a new schedule replaces the work lists the capture reads
        b.set_schedule(not persistent, 16, 16)
        with pytest.raises(bi.IntpError):
            g.launch()
    finally:
        g.close()
