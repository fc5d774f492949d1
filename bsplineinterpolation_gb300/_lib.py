"""ctypes binding of the CUDA library's C-ABI (include/intp_gpu.h).

The shared library is built in-tree by bsplineinterpolation_gb300/build.py.
There is no CPU fallback: importing the binding without the built library
raises, and every call that fails raises with the library's error message.
"""
import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libintp_gb300.so")

MAX_DIM = 4
MAX_ORDER = 7
MAX_DERIV = 16

OK = 0
ERR_INVALID_ARGUMENT = 1
ERR_DOMAIN = 2
ERR_OUT_OF_MEMORY = 3
ERR_CUDA = 4
ERR_STATE = 5
ERR_UNSUPPORTED = 6
ERR_TIMEOUT = 7
ERR_BUDGET = 8

PRECISION_FP64 = 0
PRECISION_MIXED = 1
F64 = 0
F32 = 1


class TableDesc(C.Structure):
    _fields_ = [
        ("dim", C.c_int32),
        ("order", C.c_int32),
        ("precision", C.c_int32),
        ("refine_steps", C.c_int32),
        ("periodic", C.c_int32 * MAX_DIM),
        ("size", C.c_int64 * MAX_DIM),
        ("range_lo", C.c_double * MAX_DIM),
        ("range_hi", C.c_double * MAX_DIM),
        ("coords", C.c_void_p * MAX_DIM),
        ("channels", C.c_int32),
        ("reserved_", C.c_int32),
    ]


class ServerConfig(C.Structure):
    _fields_ = [
        ("memory_budget", C.c_uint64),
        ("slots", C.c_int32),
        ("pad_", C.c_int32),
        ("max_batch_points", C.c_int64),
    ]


class ServerStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("builds_done", "evals_done", "failed", "evictions", "merged_units",
                                         "resident_tables")] + \
               [(n, C.c_uint64) for n in ("resident_bytes", "inflight_bytes")] + \
               [(n, C.c_double) for n in ("points_evaluated", "build_p50_ms", "build_p99_ms", "eval_p50_ms",
                                          "eval_p99_ms", "all_p50_ms", "all_p99_ms", "points_per_s")]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class BatchSchedule(C.Structure):
    """intp_batch_schedule."""
    _fields_ = [("persistent", C.c_int32), ("contig_rows", C.c_int32), ("strided_rows", C.c_int32),
                ("pad_", C.c_int32), ("build_ms", C.c_double)]

    def as_dict(self):
        return {"persistent": self.persistent, "contig_rows": self.contig_rows, "strided_rows": self.strided_rows,
                "build_ms": self.build_ms}


class IntpError(RuntimeError):
    """Failure reported by the CUDA library (status code and message)."""

    def __init__(self, status, msg):
        super().__init__("intp status %d: %s" % (status, msg))
        self.status = status


class IntpDomainError(IntpError, ValueError):
    """A coordinate lies outside the range of a non-periodic axis
    (the reference throws std::domain_error, Interpolation.hpp:482-491)."""


# the symbols of include/intp_gpu.h: name -> (restype, argtypes)
_P = C.c_void_p
SIGNATURES = {
    "intp_table_create": (C.c_int, [C.POINTER(TableDesc), C.POINTER(C.c_void_p)]),
    "intp_table_destroy": (C.c_int, [_P]),
    "intp_table_interpolate": (C.c_int, [_P, _P, C.c_int32, _P]),
    "intp_table_set_control_points": (C.c_int, [_P, _P]),
    "intp_table_get_control_points": (C.c_int, [_P, _P]),
    "intp_table_axis_info": (C.c_int, [_P, C.c_int32, _P, _P, _P, _P, _P]),
    "intp_table_knots": (C.c_int, [_P, C.c_int32, _P]),
    "intp_eval": (C.c_int, [_P, _P, C.c_int64, _P, C.c_int32, _P, C.c_int32, _P]),
    "intp_eval_host": (C.c_int, [_P, _P, C.c_int64, _P, C.c_int32, _P, C.c_int32, _P]),
    "intp_eval_noalloc": (C.c_int, [_P, _P, C.c_int64, _P, C.c_int32, _P, C.c_int32, _P]),
    "intp_check_range": (C.c_int, [_P, _P, C.c_int64, _P, _P]),
    "intp_locate": (C.c_int, [_P, _P, C.c_int64, _P, _P, _P]),
    "intp_locate_binned": (C.c_int, [_P, _P, C.c_int64, _P, _P]),
    "intp_stream_synchronize": (C.c_int, [_P]),
    "intp_host_alloc": (C.c_int, [C.c_size_t, C.POINTER(C.c_void_p)]),
    "intp_proxy_create": (C.c_int, [_P, _P, C.c_int64, _P, C.POINTER(C.c_void_p)]),
    "intp_proxy_destroy": (C.c_int, [_P]),
    "intp_proxy_eval": (C.c_int, [_P, _P, C.c_int32, _P, C.c_int32, _P]),
    "intp_host_free": (C.c_int, [_P]),
    "intp_debug_set_wait_limit": (C.c_int, [C.c_uint32]),
    "intp_debug_fail_allocations": (C.c_int, [C.c_int32]),
    "intp_debug_set_segment_warmup": (C.c_int, [C.c_int32]),
    "intp_last_error": (C.c_char_p, []),
    "intp_launch_count": (C.c_uint64, []),
    "intp_bandlu_create": (C.c_int, [C.c_int64, C.c_int32, C.c_int32, C.c_int32, _P, _P, _P,
                                     C.POINTER(C.c_void_p)]),
    "intp_bandlu_solve": (C.c_int, [_P, _P, C.c_int64, C.c_int64, _P]),
    "intp_bandlu_destroy": (C.c_int, [_P]),
    "intp_batch_create": (C.c_int, [C.POINTER(TableDesc), C.c_int64, C.POINTER(C.c_void_p)]),
    "intp_batch_destroy": (C.c_int, [_P]),
    "intp_batch_info": (C.c_int, [_P, _P, _P]),
    "intp_batch_build": (C.c_int, [_P, _P, C.c_int32, _P]),
    "intp_batch_get_control_points": (C.c_int, [_P, C.c_int64, _P]),
    "intp_batch_set_schedule": (C.c_int, [_P, C.POINTER(BatchSchedule)]),
    "intp_batch_get_schedule": (C.c_int, [_P, C.POINTER(BatchSchedule)]),
    "intp_batch_autotune": (C.c_int, [_P, _P, C.c_int32, _P, C.POINTER(BatchSchedule)]),
    "intp_batch_eval": (C.c_int, [_P, _P, _P, _P, C.c_int32, _P, C.c_int32, _P]),
    "intp_batch_graph_create": (C.c_int, [_P, _P, _P, _P, _P, C.c_int32, _P, C.c_int32, _P]),
    "intp_batch_graph_launch": (C.c_int, [_P, _P]),
    "intp_batch_graph_destroy": (C.c_int, [_P]),
    "intp_server_create": (C.c_int, [C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]),
    "intp_server_destroy": (C.c_int, [_P]),
    "intp_server_submit_build": (C.c_int, [_P, C.POINTER(TableDesc), _P, C.POINTER(C.c_int64),
                                           C.POINTER(C.c_int64)]),
    "intp_server_submit_eval": (C.c_int, [_P, C.c_int64, _P, C.c_int64, _P, C.c_int32, _P, C.c_int32,
                                          C.POINTER(C.c_int64)]),
    "intp_server_wait": (C.c_int, [_P, C.c_int64, C.c_double, C.POINTER(C.c_int)]),
    "intp_server_release": (C.c_int, [_P, C.c_int64]),
    "intp_server_table_state": (C.c_int, [_P, C.c_int64, C.POINTER(C.c_int32)]),
    "intp_server_get_stats": (C.c_int, [_P, C.POINTER(ServerStats)]),
    "intp_server_reset_stats": (C.c_int, [_P]),
}

_lib = None


def load():
    """Loads the built library (it must exist; nothing falls back to the CPU)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError("CUDA library %s is not built; run bsplineinterpolation_gb300.build.build()"
                          % LIB_PATH)
    lib = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status):
    if status != OK:
        msg = load().intp_last_error().decode(errors="replace")
        if status == ERR_DOMAIN:
            raise IntpDomainError(status, msg)
        raise IntpError(status, msg)
