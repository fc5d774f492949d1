"""The two evaluation paths of the mixed form -- direct (one thread per query,
gathers through L1/L2) and binned (counting sort by spatial bucket, shared-
memory tiles) -- give the same results, against each other and against the
reference's FP64 outputs, across chunk boundaries and bucket edge cases."""
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bsplineinterpolation_gb300 as bi
from tests.golden_cases import ref_outputs
from tests.gpu_util import norm_rel_err

pytestmark = pytest.mark.gpu

Z, INDEX = ref_outputs()
SMALL = [m for m in INDEX if m["dim"] <= 3]


class _Env:
    def __init__(self, **kv):
        self.kv = kv

    def __enter__(self):
        self.old = {k: os.environ.get(k) for k in self.kv}
        os.environ.update({k: str(v) for k, v in self.kv.items()})

    def __exit__(self, *a):
        for k, v in self.old.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v


def _table(meta):
    name = meta["name"]
    ranges = [Z[name + "/coords%d" % d] if meta["nonuniform"][d] else (meta["lo"][d], meta["hi"][d])
              for d in range(meta["dim"])]
    mesh = Z[name + "/values"].reshape(meta["sizes"])
    return bi.InterpolationFunction(meta["order"], meta["periodic"], torch.tensor(mesh, device="cuda"),
                                    *ranges, precision="mixed")


def _close(a, b, rel=2e-7):
    scale = np.maximum(np.max(np.abs(a), axis=0), 1e-300)
    return bool(np.all(np.abs(a - b) <= rel * scale))


def _pair_tolerance(meta):
    """Two FP32 evaluations of the same query that round differently (the
    kernels may fuse multiply-adds differently) each sit within the mixed
    form's bound 1e-6 * max(1, kappa) of the FP64 result, relative to the
    output's scale; so they agree to twice that. Derivative columns reach
    it: their weights are large and cancel (d2/dy2 on a 64-point grid of
    [0, 2] scales the weights by ~1e3)."""
    name = meta["name"]
    kappa = float(np.max(np.abs(Z[name + "/ctrl"])) / np.max(np.abs(Z[name + "/values"])))
    return 2e-6 * max(1.0, kappa)


def _eval(f, pts, derivs, mode, chunk=None):
    env = {"INTP_GB300_EVAL": mode}
    if chunk:
        env["INTP_GB300_CHUNK"] = chunk
    with _Env(**env):
        out = f.evaluate(pts, derivs=derivs)
        torch.cuda.synchronize()
    return out.double().cpu().numpy()


@pytest.mark.parametrize("meta", SMALL, ids=lambda m: m["name"])
def test_binned_equals_direct(meta):
    name = meta["name"]
    f = _table(meta)
    pts = torch.tensor(Z[name + "/points"], device="cuda")
    derivs = Z[name + "/derivs"].tolist()
    a = _eval(f, pts, derivs, "direct")
    b = _eval(f, pts, derivs, "binned")
    # same per-query code, operands from a shared-memory tile instead of L1
    assert _close(a, b, _pair_tolerance(meta))
    c = _eval(f, pts, derivs, "binned", chunk=1024)
    assert np.array_equal(b, c)


@pytest.mark.parametrize("meta", [m for m in SMALL if m["name"] in ("cube_3d_o3_20", "plain_2d_o3_64x64",
                                                                     "periodic_2d_o7_48x40")],
                         ids=lambda m: m["name"])
def test_binned_large_batch_against_reference(meta):
    """Fixture points repeated to a large shuffled batch (several chunks)."""
    name = meta["name"]
    f = _table(meta)
    base = Z[name + "/points"]
    rep = int(np.ceil(600_000 / base.shape[0]))
    perm = np.random.default_rng(3).permutation(base.shape[0] * rep)
    pts_np = np.tile(base, (rep, 1))[perm]
    want = np.tile(Z[name + "/value"], rep)[perm]
    got = _eval(f, torch.tensor(pts_np, device="cuda"), None, "binned", chunk=1 << 17)[:, 0]
    direct = _eval(f, torch.tensor(pts_np, device="cuda"), None, "direct")[:, 0]
    assert _close(got[:, None], direct[:, None], _pair_tolerance(meta))
    rng_ = Z[name + "/range"]
    inside = np.ones(pts_np.shape[0], bool)
    for d in range(meta["dim"]):
        if not meta["periodic"][d]:
            inside &= (pts_np[:, d] >= rng_[d, 0]) & (pts_np[:, d] <= rng_[d, 1])
    assert norm_rel_err(got[inside], want[inside]) < 1e-6


def test_binned_single_bucket_and_empty():
    n = 40
    g = np.linspace(-1, 1, n)
    v = np.sin(3 * g)[:, None, None] * np.cos(2 * g)[None, :, None] * g[None, None, :]
    f = bi.InterpolationFunction(3, [False] * 3, torch.tensor(v, device="cuda"), (-1, 1), (-1, 1), (-1, 1),
                                 precision="mixed")
    # every query in the same span
    pts = torch.full((300_000, 3), 0.123, dtype=torch.float64, device="cuda")
    pts[:, 1] = 0.456
    a = _eval(f, pts, [[0, 0, 0], [1, 0, 0]], "binned")
    b = _eval(f, pts[:1], [[0, 0, 0], [1, 0, 0]], "direct")
    assert _close(a, np.repeat(b, 300_000, axis=0))
    empty = torch.empty((0, 3), dtype=torch.float64, device="cuda")
    assert _eval(f, empty, None, "binned").shape == (0, 1)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_host_buffer_pipeline_equals_device_path(precision):
    """intp_eval_host with many chunks (copies in and out on their own
    streams, overlapping the evaluation of the neighbouring chunks) returns
    exactly what one device-buffer evaluation returns."""
    n = 40
    g = np.linspace(-1, 1, n)
    v = np.sin(3 * g)[:, None, None] * np.cos(2 * g)[None, :, None] * np.exp(g)[None, None, :]
    f = bi.InterpolationFunction(3, [False] * 3, torch.tensor(v, device="cuda"), (-1, 1), (-1, 1), (-1, 1),
                                 precision=precision)
    pts = np.random.default_rng(4).uniform(-1, 1, (50_003, 3))
    derivs = [[0, 0, 0], [0, 1, 0]]
    with _Env(INTP_GB300_CHUNK=4096, INTP_GB300_EVAL="direct"):
        host = f.evaluate(pts, derivs=derivs)
        dev = f.evaluate(torch.tensor(pts, device="cuda"), derivs=derivs).cpu().numpy()
    assert np.array_equal(host, dev)


def test_host_alloc_pipeline_with_growing_chunks():
    """intp_eval_host on page-locked buffers from intp_host_alloc, with a
    batch large enough for the pipeline's chunks (2^21 points, then two of
    about 2.45M for 7M points; no chunk below 2^21): every chunk takes the
    binned path and the results equal one device-buffer evaluation bit for
    bit."""
    import ctypes as C
    from bsplineinterpolation_gb300 import _lib
    lib = _lib.load()
    n = 48
    g = np.linspace(-1, 1, n)
    v = np.exp(-g)[:, None, None] * np.cos(3 * g)[None, :, None] * np.sin(2 * g + 0.3)[None, None, :]
    f = bi.InterpolationFunction(3, [False] * 3, torch.tensor(v, device="cuda"), (-1, 1), (-1, 1), (-1, 1),
                                 precision="mixed")
    npts = 7_000_000
    hp = bi.host_empty((npts, 3))
    hp[:] = np.random.default_rng(11).uniform(-1, 1, (npts, 3))
    ho = bi.host_empty((npts, 2), np.float32)
    karr = np.ascontiguousarray([[0, 0, 0], [1, 0, 0]], np.int32)
    _lib.check(lib.intp_eval_host(f._h, C.c_void_p(hp.ctypes.data), npts, karr.ctypes.data, 2,
                                  C.c_void_p(ho.ctypes.data), 1, None))
    dev = f.evaluate(torch.tensor(hp, device="cuda"), derivs=[[0, 0, 0], [1, 0, 0]]).cpu().numpy()
    assert np.array_equal(ho, dev)
