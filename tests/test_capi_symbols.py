"""The C-ABI library loads without a GPU and exports every function that
include/intp_gpu.h declares; calls that need no device fail cleanly."""
import ctypes as C
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(REPO, "include", "intp_gpu.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(intp_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from bsplineinterpolation_gb300 import _lib, build
    if not os.path.exists(_lib.LIB_PATH):
        build.build()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 15
    for name in names:
        assert hasattr(lib, name), name


def test_binding_covers_header(lib):
    from bsplineinterpolation_gb300 import _lib
    assert set(declared_functions()) == set(_lib.SIGNATURES)


def test_invalid_arguments_fail_cleanly(lib):
    from bsplineinterpolation_gb300 import _lib
    h = C.c_void_p()
    assert lib.intp_table_create(None, C.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    d = _lib.TableDesc()
    d.dim = 5
    assert lib.intp_table_create(C.byref(d), C.byref(h)) == _lib.ERR_UNSUPPORTED
    d.dim, d.order = 2, 9
    assert lib.intp_table_create(C.byref(d), C.byref(h)) == _lib.ERR_UNSUPPORTED
    d.order = 3
    d.size[0] = d.size[1] = 8
    d.range_lo[0], d.range_hi[0] = 1.0, 0.0  # decreasing range
    d.range_lo[1], d.range_hi[1] = 0.0, 1.0
    assert lib.intp_table_create(C.byref(d), C.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    assert b"increasing" in lib.intp_last_error()
    assert lib.intp_eval(None, None, 0, None, 0, None, 0, None) == _lib.ERR_INVALID_ARGUMENT
    assert lib.intp_launch_count() == 0


def test_batch_rejects_invalid_tables_before_any_device_work(lib):
    """intp_batch_create validates every descriptor on the host first."""
    from bsplineinterpolation_gb300 import _lib
    h = C.c_void_p()
    descs = (_lib.TableDesc * 3)()
    for d in descs:
        d.dim, d.order, d.precision = 1, 3, _lib.PRECISION_MIXED
        d.size[0] = 16
        d.range_lo[0], d.range_hi[0] = 0.0, 1.0
    assert lib.intp_batch_create(None, 3, C.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    assert lib.intp_batch_create(descs, 0, C.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    descs[1].dim = 4  # batched tables have dimension 1..3
    assert lib.intp_batch_create(descs, 3, C.byref(h)) == _lib.ERR_UNSUPPORTED
    assert b"table 1" in lib.intp_last_error()
    descs[1].dim = 1
    descs[2].precision = _lib.PRECISION_FP64  # one precision per batch
    assert lib.intp_batch_create(descs, 3, C.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    descs[2].precision = _lib.PRECISION_MIXED
    descs[0].size[0] = 2  # fewer samples than order + 1
    assert lib.intp_batch_create(descs, 3, C.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    assert lib.intp_launch_count() == 0


def test_server_without_a_device_fails_cleanly(lib):
    """Creating the serving loop needs CUDA streams: without a GPU it reports
    a CUDA error and leaks no worker thread."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from bsplineinterpolation_gb300 import _lib
    h = C.c_void_p()
    cfg = _lib.ServerConfig()
    cfg.slots = 65
    assert lib.intp_server_create(C.byref(cfg), C.byref(h)) == _lib.ERR_INVALID_ARGUMENT
    cfg.slots = 2
    assert lib.intp_server_create(C.byref(cfg), C.byref(h)) == _lib.ERR_CUDA
    assert not h.value
    assert lib.intp_server_destroy(None) == _lib.OK


def test_product_never_loads_the_oracle():
    """The package imports nothing from oracle/ (it is test infrastructure)."""
    pkg = os.path.join(REPO, "bsplineinterpolation_gb300")
    for root, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp", ".hpp", ".h")):
                text = open(os.path.join(root, f), errors="replace").read()
                assert "oracle" not in text.lower(), f
