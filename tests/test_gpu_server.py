"""Serving loop (intp_server_*): continuous batching, memory budget, LRU
eviction.

The central property: every request's result is the same whether it runs
alone or in a mix of concurrent builds and merged evaluations. Merged
evaluations run through one intp_eval whose per-point arithmetic does not
depend on the other points. The one difference a merge can make is to move a
request between the direct and the binned kernel (the merged size crosses the
binning threshold), and those two agree within 2e-6 of each output's scale;
the test holds results to that tolerance.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bsplineinterpolation_gb300 as bi
from oracle import oracle
from tests.gpu_util import norm_rel_err

pytestmark = pytest.mark.gpu

# every wait is bounded: a request that never completes fails the test
# instead of stalling the run
WAIT_S = 120.0

OK = 0
ERR_STATE = 5
ERR_BUDGET = 8


def _smooth(rng, dims):
    axes = [np.linspace(0.0, 1.0, n) for n in dims]
    grids = np.meshgrid(*axes, indexing="ij")
    f = np.ones(dims)
    for g in grids:
        f = f * np.cos(rng.uniform(1, 4) * g + rng.uniform(0, 2 * np.pi))
    return f + 1e-3 * rng.normal(size=dims)


TABLES = [  # (order, periodicity, dims)
    (3, [False, False], [48, 40]),
    (5, [True, True], [64, 64]),
    (3, [False, False, False], [24, 20, 28]),
    (5, [False], [300]),
    (3, [True, False], [128, 96]),
]


def _pinned(a):
    return torch.from_numpy(np.ascontiguousarray(a)).pin_memory()


def _build_all(srv, rng):
    ids, data = [], []
    for order, per, dims in TABLES:
        vals = _pinned(_smooth(rng, dims))
        tid, rid = srv.submit_build(order, per, vals, *[(0.0, 1.0)] * len(dims))
        ids.append((tid, rid))
        data.append(vals)
    for tid, rid in ids:
        assert srv.wait(rid, WAIT_S) == OK
        assert srv.table_state(tid) == "resident"
    return [tid for tid, _ in ids], data


def _requests(rng, ids, n):
    reqs = []
    for _ in range(n):
        k = int(rng.integers(len(TABLES)))
        D = len(TABLES[k][2])
        npts = int(np.exp(rng.uniform(np.log(10), np.log(400_000))))
        pts = _pinned(rng.uniform(0.0, 1.0, (npts, D)))
        derivs = None
        if rng.random() < 0.4:
            d = np.zeros((2, D), np.int32)
            d[1, 0] = 1
            derivs = d
        reqs.append((ids[k], pts, derivs))
    return reqs


def _out_for(pts, derivs):
    K = 1 if derivs is None else derivs.shape[0]
    return torch.empty((pts.shape[0], K), dtype=torch.float32).pin_memory()


def test_results_same_alone_and_in_the_mix():
    rng = np.random.default_rng(20261207)
    srv = bi.Server(slots=4)
    try:
        ids, data = _build_all(srv, rng)
        reqs = _requests(rng, ids, 40)
        alone = []
        for tid, pts, derivs in reqs:
            out = _out_for(pts, derivs)
            assert srv.wait(srv.submit_eval(tid, pts, out, derivs), WAIT_S) == OK
            alone.append(out.numpy().copy())
        # the mix: every evaluation at once, with new builds interleaved
        outs, rids, extra = [], [], []
        for i, (tid, pts, derivs) in enumerate(reqs):
            out = _out_for(pts, derivs)
            outs.append(out)
            rids.append(srv.submit_eval(tid, pts, out, derivs))
            if i % 10 == 5:
                order, per, dims = TABLES[i % len(TABLES)]
                vals = _pinned(_smooth(rng, [2 * d for d in dims]))
                extra.append((vals,) + srv.submit_build(order, per, vals, *[(0.0, 1.0)] * len(dims)))
        for rid in rids:
            assert srv.wait(rid, WAIT_S) == OK
        for _, tid, rid in extra:
            assert srv.wait(rid, WAIT_S) == OK
        for a, b in zip(alone, outs):
            b = b.numpy()
            scale = np.maximum(np.max(np.abs(a), axis=0), 1e-30)
            assert np.all(np.abs(a - b) <= 2e-6 * scale)
        st = srv.stats()
        assert st["failed"] == 0 and st["evals_done"] == 80
    finally:
        srv.close()


def test_served_table_matches_oracle_and_direct_table():
    rng = np.random.default_rng(11)
    srv = bi.Server(slots=2)
    try:
        order, per, dims = TABLES[2]
        vals_np = _smooth(rng, dims)
        tid, rid = srv.submit_build(order, per, _pinned(vals_np), *[(0.0, 1.0)] * 3)
        assert srv.wait(rid, WAIT_S) == OK
        pts = _pinned(rng.uniform(0.0, 1.0, (5000, 3)))
        out = _out_for(pts, None)
        assert srv.wait(srv.submit_eval(tid, pts, out), WAIT_S) == OK
        ref = oracle.Spline(3, order, per, dims, [0.0] * 3, [1.0] * 3).interpolate(vals_np)
        assert norm_rel_err(out.numpy()[:, 0], ref.eval(pts.numpy())) < 1e-6
        f = bi.InterpolationFunction(order, per, torch.tensor(vals_np, device="cuda"), *[(0.0, 1.0)] * 3,
                                     precision="mixed")
        assert np.array_equal(f.evaluate(pts.numpy()), out.numpy())
    finally:
        srv.close()


def test_budget_and_lru_eviction():
    """2D 1024^2 mixed tables hold 8 MiB each (their control points as two
    FP32 arrays); a build needs ~25 MiB in flight (the table and 16 bytes of
    scratch per value: the staged values and the double-word solve's working
    array). Under a 60 MiB budget five tables fit with a build in flight
    and the sixth build evicts the least recently used idle table; an
    evaluation of an evicted table reports ERR_STATE and a request that
    could never fit reports ERR_BUDGET."""
    rng = np.random.default_rng(5)
    srv = bi.Server(memory_budget=60 << 20, slots=1)
    try:
        vals = [_pinned(_smooth(rng, [1024, 1024])) for _ in range(7)]
        tids = []
        for i in range(5):
            tid, rid = srv.submit_build(3, [False, False], vals[i], (0.0, 1.0), (0.0, 1.0))
            assert srv.wait(rid, WAIT_S) == OK
            tids.append(tid)
        assert all(srv.table_state(t) == "resident" for t in tids)
        # touch table 0: table 1 becomes the least recently used
        pts = _pinned(rng.uniform(0.0, 1.0, (1000, 2)))
        out = _out_for(pts, None)
        assert srv.wait(srv.submit_eval(tids[0], pts, out), WAIT_S) == OK
        tid5, rid = srv.submit_build(3, [False, False], vals[5], (0.0, 1.0), (0.0, 1.0))
        assert srv.wait(rid, WAIT_S) == OK
        assert srv.table_state(tids[1]) == "gone"
        assert srv.table_state(tids[0]) == "resident"
        assert srv.stats()["evictions"] == 1
        assert srv.wait(srv.submit_eval(tids[1], pts, out), WAIT_S) == ERR_STATE
        assert srv.wait(srv.submit_eval(tid5, pts, out), WAIT_S) == OK
        big = _pinned(_smooth(rng, [2048, 2048]))
        _, rid = srv.submit_build(3, [False, False], big, (0.0, 1.0), (0.0, 1.0))
        assert srv.wait(rid, WAIT_S) == ERR_BUDGET
        assert srv.stats()["resident_bytes"] <= 60 << 20
    finally:
        srv.close()


def test_queued_evaluations_merge():
    """With one slot busy on a build, evaluations queued behind it against
    the same table are merged into one work unit, and each still gets its own
    results."""
    rng = np.random.default_rng(9)
    srv = bi.Server(slots=1)
    try:
        order, per, dims = TABLES[0]
        vals_np = _smooth(rng, dims)
        tid, rid0 = srv.submit_build(order, per, _pinned(vals_np), *[(0.0, 1.0)] * 2)
        reqs = []
        for _ in range(12):
            pts = _pinned(rng.uniform(0.0, 1.0, (int(rng.integers(1, 5000)), 2)))
            out = _out_for(pts, None)
            reqs.append((pts, out, srv.submit_eval(tid, pts, out)))
        assert srv.wait(rid0, WAIT_S) == OK
        for _, _, rid in reqs:
            assert srv.wait(rid, WAIT_S) == OK
        assert srv.stats()["merged_units"] >= 1
        ref = oracle.Spline(2, order, per, dims, [0.0] * 2, [1.0] * 2).interpolate(vals_np)
        for pts, out, _ in reqs:
            assert norm_rel_err(out.numpy()[:, 0], ref.eval(pts.numpy())) < 1e-6
    finally:
        srv.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_vector_valued_table_served(precision):
    """A C-channel table (the reference's InterpolationFunction with a vector
    T) built and evaluated through the server gives what the same table built
    and evaluated directly gives, bit for bit, and each channel agrees with
    the oracle's scalar table of that channel."""
    rng = np.random.default_rng(31)
    order, per, dims, C = 3, [False, True], [40, 36], 3
    vals_np = np.stack([_smooth(rng, dims) for _ in range(C)], axis=-1)
    ranges = [(0.0, 1.0)] * 2
    srv = bi.Server(slots=2)
    try:
        tid, rid = srv.submit_build(order, per, _pinned(vals_np), *ranges, precision=precision, vector=True)
        assert srv.wait(rid, WAIT_S) == OK
        pts_np = rng.uniform(0.0, 1.0, (4000, 2))
        derivs = np.array([[0, 0], [0, 1]], np.int32)
        pts = _pinned(pts_np)
        out = torch.empty((4000, 2, C), dtype=torch.float64).pin_memory()
        assert srv.wait(srv.submit_eval(tid, pts, out, derivs=derivs, out_dtype="f64"), WAIT_S) == OK
        f = bi.InterpolationFunction(order, per, vals_np, *ranges, precision=precision, vector=True)
        want = f.evaluate(torch.tensor(pts_np, device="cuda"), derivs=derivs, out_dtype="f64").cpu().numpy()
        assert np.array_equal(out.numpy(), want)
        tol = 1e-12 if precision == "fp64" else 1e-6
        for c in range(C):
            ref = oracle.Spline(2, order, per, dims, [0.0] * 2, [1.0] * 2).interpolate(vals_np[..., c])
            assert norm_rel_err(out.numpy()[:, 0, c], ref.eval(pts_np)) < tol
    finally:
        srv.close()
