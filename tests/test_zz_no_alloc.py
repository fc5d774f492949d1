"""The allocation-free evaluation entry point, intp_eval_noalloc, called
through the C-ABI on the GPU: against the regular entry point intp_eval and
against the oracle, on two calls in a row, and with no device allocation
during a call.

Some callers cannot allocate device memory during evaluation: a host that has
already handed all of the GPU's memory to its own pool, or a latency-bound
loop where cudaMalloc's implicit synchronisation is not acceptable. For them
intp_eval_noalloc takes its scratch from one fixed 8 MiB device array inside
the library instead of allocating. This file is collected last so that a run
that stops at its first failure has already run every other test; it also
passes on its own in a fresh process (the first call sets the array up)."""
import ctypes as C
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bsplineinterpolation_gb300 as bi
from bsplineinterpolation_gb300 import _lib
from oracle import oracle

pytestmark = pytest.mark.gpu

TOL = 2e-7  # FP32 ulps of each output's scale, as the evaluation-path tests use


def _grid3(n):
    g = np.linspace(-1, 1, n)
    return np.exp(-(g[:, None, None] ** 2 + g[None, :, None] ** 2 + g[None, None, :] ** 2)) * np.cos(4 * g)[:, None, None]


def _table3():
    v = _grid3(96)
    return bi.InterpolationFunction(3, [False] * 3, torch.tensor(v, device="cuda"), (-1, 1), (-1, 1), (-1, 1),
                                    precision="mixed"), v


def _table2_periodic():
    # periodic in both axes: bucket tiles that wrap an axis are staged with
    # element copies (the TMA box cannot wrap)
    n0, n1 = 200, 150
    x = np.arange(n0) * (2 * np.pi / n0)
    y = np.arange(n1) * (2 * np.pi / n1)
    v = np.sin(3 * x)[:, None] * np.cos(2 * y)[None, :] + 0.3 * np.cos(x[:, None] + 4 * y[None, :])
    r = (0.0, 2 * np.pi)
    return bi.InterpolationFunction(5, [True, True], torch.tensor(v, device="cuda"), r, r, precision="mixed"), v


def _call(fn, f, pts, derivs):
    lib = _lib.load()
    k = np.ascontiguousarray(derivs, np.int32)
    out = torch.empty((pts.shape[0], k.shape[0]), dtype=torch.float32, device="cuda")
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    _lib.check(getattr(lib, fn)(f._h, C.c_void_p(pts.data_ptr()), pts.shape[0], k.ctypes.data, k.shape[0],
                                C.c_void_p(out.data_ptr()), _lib.F32, stream))
    torch.cuda.synchronize()
    return out.double().cpu().numpy()


def _close(a, b, tol=TOL):
    scale = np.maximum(np.max(np.abs(a), axis=0), 1e-300)
    return bool(np.all(np.abs(a - b) <= tol * scale))


def _oracle_err(ref, pts, derivs, got):
    want = ref.derivative(pts.cpu().numpy(), derivs, nthreads=os.cpu_count() or 1)
    return max(float(np.max(np.abs(got[:, k] - want[:, k])) / np.max(np.abs(want[:, k])))
               for k in range(len(derivs)))


def test_noalloc_matches_regular_entry_point_twice():
    f, v = _table3()
    ref = oracle.Spline(3, 3, [False] * 3, [96] * 3, [-1.0] * 3, [1.0] * 3).interpolate(v)
    derivs = [[0, 0, 0], [1, 0, 0], [0, 2, 1]]
    gen = torch.Generator(device="cuda")
    gen.manual_seed(7)
    # more queries than one pass over the fixed area holds: several chunks
    for npts in (1_500_000, 700_000):
        pts = torch.rand((npts, 3), dtype=torch.float64, device="cuda", generator=gen) * 2 - 1
        want = _call("intp_eval", f, pts, derivs)
        got = _call("intp_eval_noalloc", f, pts, derivs)
        assert _close(want, got)
        # and against the oracle (the reference algorithm in FP64): the mixed
        # form's bound for values and first derivatives, 1e-6 of each
        # output's scale
        assert _oracle_err(ref, pts[:200_000], derivs[:2], got[:200_000, :2]) < 1e-6


def test_noalloc_periodic_2d_twice():
    f, v = _table2_periodic()
    ref = oracle.Spline(2, 5, [True, True], list(v.shape), [0.0, 0.0], [2 * np.pi] * 2).interpolate(v)
    derivs = [[0, 0], [1, 0], [0, 1]]
    gen = torch.Generator(device="cuda")
    gen.manual_seed(11)
    for npts in (600_000, 2_000_000):
        # points over three periods: every query wraps
        pts = (torch.rand((npts, 2), dtype=torch.float64, device="cuda", generator=gen) * 3 - 1) * (2 * np.pi)
        want = _call("intp_eval", f, pts, derivs)
        got = _call("intp_eval_noalloc", f, pts, derivs)
        assert _close(want, got)
        assert _oracle_err(ref, pts[:200_000], derivs, got[:200_000]) < 1e-6


def _cudart():
    for name in ("libcudart.so", "libcudart.so.13", "/usr/local/cuda/lib64/libcudart.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    return None


def test_noalloc_allocates_nothing():
    """Neither the device's default memory pool (the stream-ordered
    allocator intp_eval uses) nor the device's free memory changes during a
    call of a few chunks."""
    f, _ = _table3()
    derivs = [[0, 0, 0], [1, 0, 0]]
    pts = torch.rand((1_200_000, 3), dtype=torch.float64, device="cuda") * 2 - 1
    _call("intp_eval_noalloc", f, pts, derivs)  # first launches load their kernels
    torch.cuda.synchronize()
    rt = _cudart()
    pool = C.c_void_p()
    if rt is not None:
        dev = torch.cuda.current_device()
        assert rt.cudaDeviceGetDefaultMemPool(C.byref(pool), dev) == 0
        zero = C.c_uint64(0)
        assert rt.cudaMemPoolSetAttribute(pool, 0x8, C.byref(zero)) == 0  # reset UsedMemHigh
        used0 = C.c_uint64()
        assert rt.cudaMemPoolGetAttribute(pool, 0x7, C.byref(used0)) == 0  # UsedMemCurrent
    free0, _ = torch.cuda.mem_get_info()
    _call("intp_eval_noalloc", f, pts, derivs)
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    if rt is not None:
        high = C.c_uint64()
        assert rt.cudaMemPoolGetAttribute(pool, 0x8, C.byref(high)) == 0
        assert high.value == used0.value


def test_noalloc_rejects_tables_beyond_its_area():
    # 512^3 spans: 32^3 buckets need more bookkeeping than the 8 MiB area
    n = 520
    v = torch.zeros((n, n, n), dtype=torch.float64, device="cuda")
    f = bi.InterpolationFunction(3, [False] * 3, v, (0, 1), (0, 1), (0, 1), precision="mixed")
    pts = torch.rand((1000, 3), dtype=torch.float64, device="cuda")
    with pytest.raises(bi.IntpError, match="too many buckets"):
        _call("intp_eval_noalloc", f, pts, [[0, 0, 0]])
