"""The allocation-free evaluation entry point, intp_eval_noalloc, against the
regular entry point intp_eval, called through the C-ABI on the GPU.

Some callers cannot allocate device memory during evaluation: a host that has
already handed all of the GPU's memory to its own pool, or a latency-bound
loop where cudaMalloc's implicit synchronisation is not acceptable. For them
intp_eval_noalloc takes its scratch from one fixed 8 MiB device array inside
the library instead of allocating. This file is collected last so that a run
that stops at its first failure has already run every other test; it also
passes on its own in a fresh process (the first call sets the array up)."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bsplineinterpolation_gb300 as bi
from bsplineinterpolation_gb300 import _lib

pytestmark = pytest.mark.gpu

TOL = 2e-7  # FP32 ulps of each output's scale, as the evaluation-path tests use


def _table():
    n = 96
    g = np.linspace(-1, 1, n)
    v = np.exp(-(g[:, None, None] ** 2 + g[None, :, None] ** 2 + g[None, None, :] ** 2)) * np.cos(4 * g)[:, None, None]
    return bi.InterpolationFunction(3, [False] * 3, torch.tensor(v, device="cuda"), (-1, 1), (-1, 1), (-1, 1),
                                    precision="mixed")


def _call(fn, f, pts, derivs):
    lib = _lib.load()
    k = np.ascontiguousarray(derivs, np.int32)
    out = torch.empty((pts.shape[0], k.shape[0]), dtype=torch.float32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(getattr(lib, fn)(f._h, C.c_void_p(pts.data_ptr()), pts.shape[0], k.ctypes.data, k.shape[0],
                                C.c_void_p(out.data_ptr()), _lib.F32, stream))
    torch.cuda.synchronize()
    return out.double().cpu().numpy()


def _close(a, b):
    scale = np.maximum(np.max(np.abs(a), axis=0), 1e-300)
    return bool(np.all(np.abs(a - b) <= TOL * scale))


def test_noalloc_matches_regular_entry_point_twice():
    f = _table()
    derivs = [[0, 0, 0], [1, 0, 0], [0, 2, 1]]
    gen = torch.Generator(device="cuda")
    gen.manual_seed(7)
    # more queries than one pass over the fixed area holds: several chunks
    for npts in (1_500_000, 700_000):
        pts = torch.rand((npts, 3), dtype=torch.float64, device="cuda", generator=gen) * 2 - 1
        want = _call("intp_eval", f, pts, derivs)
        got = _call("intp_eval_noalloc", f, pts, derivs)
        assert _close(want, got)


def test_noalloc_rejects_tables_beyond_its_area():
    # 512^3 spans: 32^3 buckets need more bookkeeping than the 8 MiB area
    n = 520
    v = torch.zeros((n, n, n), dtype=torch.float64, device="cuda")
    f = bi.InterpolationFunction(3, [False] * 3, v, (0, 1), (0, 1), (0, 1), precision="mixed")
    pts = torch.rand((1000, 3), dtype=torch.float64, device="cuda")
    with pytest.raises(bi.IntpError, match="too many buckets"):
        _call("intp_eval_noalloc", f, pts, [[0, 0, 0]])
