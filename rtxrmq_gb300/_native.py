"""ctypes binding of librmq.so (the C ABI declared in include/rmq.h).

The library is the only compute path: if it has not been built, importing
``lib`` raises, there is no Python or CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "librmq.so"

RMQ_OK = 0
RMQ_EINVAL = -1
RMQ_ENOMEM = -2
RMQ_ECUDA = -3
RMQ_ENOTSUP = -5

_STATUS_NAMES = {RMQ_EINVAL: "RMQ_EINVAL", RMQ_ENOMEM: "RMQ_ENOMEM", RMQ_ECUDA: "RMQ_ECUDA",
                 RMQ_ENOTSUP: "RMQ_ENOTSUP"}


class RMQError(RuntimeError):
    """A C-ABI call returned a negative status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{_STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class rmq_info_t(C.Structure):
    _fields_ = [("n", C.c_int64), ("bs", C.c_int64), ("nb", C.c_int64), ("levels", C.c_int32),
                ("aligned", C.c_int32), ("table_bytes", C.c_int64), ("struct_bytes", C.c_int64),
                ("micro_levels", C.c_int32), ("light", C.c_int32),
                ("micro_table_bytes", C.c_int64), ("is_max", C.c_int32), ("is_int32", C.c_int32)]

RMQ_BUILD_NO_MICRO = 1
RMQ_BUILD_MAX = 2
RMQ_BUILD_INT32 = 4
RMQ_BUILD_LIGHT = 8


RMQ_BATCH_BUCKETS = 32


class rmq_batch_info_t(C.Structure):
    _fields_ = [("narrays", C.c_int32), ("max_levels", C.c_int32), ("values_span", C.c_int64),
                ("queries_span", C.c_int64), ("workspace_bytes", C.c_int64),
                ("device_bytes", C.c_int64), ("build_items", C.c_int32),
                ("query_items", C.c_int32), ("bucket_bs", C.c_int32 * RMQ_BATCH_BUCKETS),
                ("flags", C.c_int32)]


class rmq_batch_tile_t(C.Structure):
    _fields_ = [("bs", C.c_int32), ("query_chunk", C.c_int32), ("level_chunk", C.c_int32),
                ("reserved", C.c_int32)]


_vp, _i64, _i32, _u64, _dbl = C.c_void_p, C.c_int64, C.c_int32, C.c_uint64, C.c_double

# name -> (restype, argtypes); every symbol include/rmq.h declares
SIGNATURES = {
    "rmq_build": (C.c_int, [_vp, _i64, _i64, _vp, C.POINTER(_vp)]),
    "rmq_build_ex": (C.c_int, [_vp, _i64, _i64, C.c_uint32, _vp, C.POINTER(_vp)]),
    "rmq_query": (C.c_int, [_vp, _vp, _i64, _vp, _vp, _vp]),
    "rmq_query_host": (C.c_int, [_vp, _vp, _i64, _vp, _vp, _vp]),
    "rmq_query_noalloc": (C.c_int, [_vp, _i64, _i64, _vp, _i64, _vp, _vp, _vp]),
    "rmq_free": (C.c_int, [_vp]),
    "rmq_save": (C.c_int, [_vp, C.c_char_p, _vp]),
    "rmq_load": (C.c_int, [_vp, _i64, C.c_char_p, _vp, C.POINTER(_vp)]),
    "rmq_info": (C.c_int, [_vp, C.POINTER(rmq_info_t)]),
    "rmq_invalid_count": (C.c_int, [_vp, _vp, C.POINTER(_i64)]),
    "rmq_last_error_string": (C.c_char_p, []),
    "rmq_version": (C.c_char_p, []),
    "rmq_bs_from_nb": (C.c_int, [_i64, _i64, C.POINTER(_i64)]),
    "rmq_query_scan": (C.c_int, [_vp, _i64, _vp, _i64, _vp, _vp, _vp]),
    "rmq_probe_gather": (C.c_int, [_vp, _vp, _i64, _vp, _vp, _vp]),
    "rmq_query_stats": (C.c_int, [_vp, _vp, _i64, _vp, _vp, C.POINTER(_i64), _vp]),
    "rmq_probe_random": (C.c_int, [_vp, _i64, _vp, _i64, _vp, _vp, _vp]),
    "rmq_checked_violations": (C.c_int, [C.POINTER(_i64)]),
    "rmq_batch_create": (C.c_int, [_i32, _vp, _vp, _vp, _vp, _vp, C.POINTER(_vp)]),
    "rmq_batch_create_ex": (C.c_int, [_i32, _vp, _vp, _vp, _vp, _vp, C.c_uint32, C.POINTER(_vp)]),
    "rmq_batch_tiles": (C.c_int, [_vp, _vp]),
    "rmq_batch_autotune_ex": (C.c_int, [_i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _vp,
                                        C.c_uint32, _vp]),
    "rmq_batch_run": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "rmq_batch_run_per_array": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "rmq_batch_build": (C.c_int, [_vp, _vp, _vp]),
    "rmq_batch_query": (C.c_int, [_vp, _vp, _vp, _vp, _vp, _vp]),
    "rmq_batch_scatter_grad": (C.c_int, [_vp, _vp, _vp, _vp, _i32, _vp]),
    "rmq_batch_info": (C.c_int, [_vp, C.POINTER(rmq_batch_info_t)]),
    "rmq_batch_invalid_count": (C.c_int, [_vp, _vp, C.POINTER(_i64)]),
    "rmq_batch_free": (C.c_int, [_vp]),
    "rmq_batch_autotune": (C.c_int, [_i32, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i32, _vp, _vp]),
    "rmq_power_begin": (C.c_int, [_i32, _i32, _i32, C.c_char_p]),
    "rmq_power_end": (C.c_int, [_i32, C.POINTER(_dbl), C.POINTER(_dbl), C.POINTER(_dbl)]),
    "rmq_gen_values_uniform": (C.c_int, [_vp, _i64, _u64]),
    "rmq_gen_values_normal": (C.c_int, [_vp, _i64, _dbl, _dbl, _u64]),
    "rmq_gen_values_int": (C.c_int, [_vp, _i64, _i32, _u64]),
    "rmq_gen_queries": (C.c_int, [_vp, _i64, _i64, _i32, _u64]),
    "rmq_gen_queries_lognormal": (C.c_int, [_vp, _i64, _i64, _dbl, _dbl, _u64]),
}

_lock = threading.Lock()
_lib: C.CDLL | None = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Load librmq.so once and attach the signatures; raise if it is missing."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise RuntimeError(
                f"{p} is missing: build the CUDA engine first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        lib = C.CDLL(str(p))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(rc: int) -> None:
    if rc != RMQ_OK:
        msg = load().rmq_last_error_string()
        raise RMQError(rc, msg.decode() if msg else "")
