"""Failure paths, driven without faulting or hanging the device.

- A bounded device wait that runs out: the binned evaluation waits for each
  staged tile on a barrier; intp_debug_set_wait_limit(1) makes that wait a
  single non-blocking probe, which gives up while the tile copy is still in
  flight. The kernel records the timeout and stops after the copy has
  landed; intp_stream_synchronize reports INTP_ERR_TIMEOUT, and the next
  evaluation with the normal wait is correct (the context stays usable).
- An allocation failure in the serving loop: intp_debug_fail_allocations(1)
  fails the next table allocation as out of memory; the build request
  reports INTP_ERR_OUT_OF_MEMORY (the reference's std::bad_alloc,
  aligned-allocator.hpp), the table is marked failed, evaluations against it
  report INTP_ERR_STATE, and the next build succeeds."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")

import bsplineinterpolation_gb300 as bi
from bsplineinterpolation_gb300 import _lib

pytestmark = pytest.mark.gpu


def _table():
    n = 96  # rows of 96 floats: 16-byte aligned, so tiles are staged by TMA
    g = np.linspace(-1, 1, n)
    v = np.exp(-(g[:, None, None] ** 2 + g[None, :, None] ** 2 + g[None, None, :] ** 2)) * np.cos(4 * g)[:, None, None]
    return bi.InterpolationFunction(3, [False] * 3, torch.tensor(v, device="cuda"), (-1, 1), (-1, 1), (-1, 1),
                                    precision="mixed")


def test_tile_wait_timeout_is_reported_and_recoverable():
    lib = _lib.load()
    f = _table()
    pts = torch.rand((1_000_000, 3), dtype=torch.float64, device="cuda") * 2 - 1
    derivs = [[0, 0, 0], [1, 0, 0]]
    want = f.evaluate(pts, derivs=derivs).double().cpu().numpy()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.intp_stream_synchronize(stream) == _lib.OK
    try:
        _lib.check(lib.intp_debug_set_wait_limit(1))
        out = torch.empty((pts.shape[0], 2), dtype=torch.float32, device="cuda")
        k = np.ascontiguousarray(derivs, np.int32)
        _lib.check(lib.intp_eval(f._h, C.c_void_p(pts.data_ptr()), pts.shape[0], k.ctypes.data, 2,
                                 C.c_void_p(out.data_ptr()), _lib.F32, stream))
        assert lib.intp_stream_synchronize(stream) == _lib.ERR_TIMEOUT
        assert b"bounded wait" in lib.intp_last_error()
    finally:
        _lib.check(lib.intp_debug_set_wait_limit(0))
    # the flag was read and cleared; the normal wait evaluates correctly
    got = f.evaluate(pts, derivs=derivs).double().cpu().numpy()
    assert lib.intp_stream_synchronize(stream) == _lib.OK
    assert np.array_equal(got, want)


def test_server_build_out_of_memory_is_reported():
    lib = _lib.load()
    srv = bi.Server(memory_budget=8 << 30, slots=2)
    try:
        v = torch.rand((64, 64, 64), dtype=torch.float64, device="cuda")
        _lib.check(lib.intp_debug_fail_allocations(1))
        try:
            tid, rid = srv.submit_build(3, [False] * 3, v, (0.0, 1.0), (0.0, 1.0), (0.0, 1.0))
            assert srv.wait(rid, 60.0) == _lib.ERR_OUT_OF_MEMORY
        finally:
            _lib.check(lib.intp_debug_fail_allocations(0))
        pts = torch.rand((1000, 3), dtype=torch.float64, device="cuda")
        out = torch.empty((1000, 1), dtype=torch.float32, device="cuda")
        assert srv.wait(srv.submit_eval(tid, pts, out), 60.0) == _lib.ERR_STATE
        tid2, rid2 = srv.submit_build(3, [False] * 3, v, (0.0, 1.0), (0.0, 1.0), (0.0, 1.0))
        assert srv.wait(rid2, 60.0) == _lib.OK
        assert srv.wait(srv.submit_eval(tid2, pts, out), 60.0) == _lib.OK
    finally:
        srv.close()
