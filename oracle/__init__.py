"""CPU oracle for the batch RMQ path -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
bench.py import this package, and only as the checker or the timed CPU
baseline; the product (librmq.so, the rtxrmq CLI, rtxrmq_gb300) never uses
it.

* ``liboracle.so`` (rmq_oracle.c): plain-C restatement of the reference's
  CPU BASE (src/cpu_methods.h:6-77) and of RTX_blocks' block decomposition
  (src/rtx_kernels.cu:85-180, src/rtx.h:3-22).
* ``_ref/libref.so`` (built only where the reference tree is present): the
  reference's own cpu_rmq / cpu_rmq_idx / rmq_rmm_par(_idx) (HRMQ) and
  random_queries_par_cpu, compiled unmodified by oracle/Makefile. Used to
  generate the golden vectors under tests/golden/ and to pin the restatement.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
REF_LIB = HERE / "_ref" / "libref.so"
# Where the build recipe below reads the reference's sources: the tree named
# by RTXRMQ_REFERENCE, else the development container's mount point. Only
# this recipe reads it; no other code of the project does.
_DEV_REFERENCE_MOUNT = "/root/reference"


def reference_tree() -> Path | None:
    """The reference tree to compile oracle/_ref from, or None when absent."""
    env = os.environ.get("RTXRMQ_REFERENCE")
    t = Path(env) if env else Path(_DEV_REFERENCE_MOUNT)
    return t if (t / "hrmq" / "RMQRMM64.cpp").exists() else None

_vp, _i64, _i32 = C.c_void_p, C.c_int64, C.c_int
_lib = None
_ref = None


def build(with_ref: bool | None = None) -> None:
    """Compile liboracle.so; with_ref=None also compiles _ref/libref.so when
    the reference tree is present, True requires it."""
    targets = ["all"]
    ref = reference_tree()
    if with_ref and ref is None:
        raise FileNotFoundError("the reference tree was not found: set RTXRMQ_REFERENCE to it")
    if with_ref is None:
        with_ref = ref is not None
    args = ["make", "-s", "-C", str(HERE)]
    if with_ref:
        targets.append("ref")
        args.append(f"REF={ref}")
    r = subprocess.run([*args, *targets], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB.exists():
            build(with_ref=False)
        L = C.CDLL(str(LIB))
        L.oracle_base_val.argtypes = [_vp, _i64, _vp, _i64, _vp, _i32]
        L.oracle_base_idx.argtypes = [_vp, _i64, _vp, _i64, _vp, _i32]
        L.oracle_blocks_build.restype = _vp
        L.oracle_blocks_build.argtypes = [_vp, _i64, _i64, _i32]
        L.oracle_blocks_query.argtypes = [_vp, _vp, _i64, _vp, _vp, _i32]
        L.oracle_blocks_free.argtypes = [_vp]
        L.oracle_max_threads.restype = _i32
        L.hrmq_port_build.restype = _vp
        L.hrmq_port_build.argtypes = [_vp, _i64, _i32, _i32]
        L.hrmq_port_query.argtypes = [_vp, _vp, _vp, _i64, _vp, _vp, _i32]
        L.hrmq_port_bytes.restype = _i64
        L.hrmq_port_bytes.argtypes = [_vp]
        L.hrmq_port_free.argtypes = [_vp]
        _lib = L
    return _lib


def _arr(a, dtype):
    a = np.ascontiguousarray(a, dtype=dtype)
    return a, a.ctypes.data


def max_threads() -> int:
    return lib().oracle_max_threads()


def base_val(A, Q, nt: int = 0) -> np.ndarray:
    """cpu_rmq restated: leftmost minimum values (float32)."""
    A, pa = _arr(A, np.float32)
    Q, pq = _arr(Q, np.int32)
    out = np.empty(len(Q), dtype=np.float32)
    if lib().oracle_base_val(pa, len(A), pq, len(Q), out.ctypes.data, nt) != 0:
        raise ValueError("oracle_base_val: bad arguments")
    return out


def base_idx(A, Q, nt: int = 0) -> np.ndarray:
    """cpu_rmq_idx restated: leftmost argmin (int32)."""
    A, pa = _arr(A, np.float32)
    Q, pq = _arr(Q, np.int32)
    out = np.empty(len(Q), dtype=np.int32)
    if lib().oracle_base_idx(pa, len(A), pq, len(Q), out.ctypes.data, nt) != 0:
        raise ValueError("oracle_base_idx: bad arguments")
    return out


class Blocks:
    """RTX_blocks restated on the CPU (block minima + partial-block scans)."""

    def __init__(self, A, bs: int, nt: int = 0):
        self.A, pa = _arr(A, np.float32)
        self._h = lib().oracle_blocks_build(pa, len(self.A), bs, nt)
        if not self._h:
            raise MemoryError("oracle_blocks_build failed")

    def query(self, Q, nt: int = 0):
        Q, pq = _arr(Q, np.int32)
        val = np.empty(len(Q), dtype=np.float32)
        idx = np.empty(len(Q), dtype=np.int32)
        if lib().oracle_blocks_query(self._h, pq, len(Q), val.ctypes.data, idx.ctypes.data,
                                     nt) != 0:
            raise ValueError("oracle_blocks_query: bad arguments")
        return val, idx

    def close(self):
        if self._h:
            lib().oracle_blocks_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class HRMQ:
    """The reference's CPU comparator HRMQ (hrmq/RMQRMM64.cpp) restated in
    hrmq_port.c: balanced-parentheses RMQ. strict=False resolves ties
    rightmost (as HRMQ), strict=True leftmost (as BASE)."""

    def __init__(self, A, strict: bool = False, nt: int = 0):
        self.A, pa = _arr(A, np.float32)
        self._h = lib().hrmq_port_build(pa, len(self.A), int(bool(strict)), nt)
        if not self._h:
            raise MemoryError("hrmq_port_build failed")

    def query(self, Q, nt: int = 0):
        Q, pq = _arr(Q, np.int32)
        val = np.empty(len(Q), dtype=np.float32)
        idx = np.empty(len(Q), dtype=np.int32)
        if lib().hrmq_port_query(self._h, self.A.ctypes.data, pq, len(Q), val.ctypes.data,
                                 idx.ctypes.data, nt) != 0:
            raise ValueError("hrmq_port_query: bad arguments")
        return val, idx

    def nbytes(self) -> int:
        return lib().hrmq_port_bytes(self._h)

    def close(self):
        if self._h:
            lib().hrmq_port_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- the reference's own CPU code (present only where the reference compiled) ----

def ref_available() -> bool:
    return REF_LIB.exists()


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            raise FileNotFoundError(f"{REF_LIB} not built (reference tree absent)")
        R = C.CDLL(str(REF_LIB))
        for name in ("ref_cpu_rmq", "ref_cpu_rmq_idx", "ref_rmq_rmm_par", "ref_rmq_rmm_par_idx"):
            getattr(R, name).argtypes = [_i32, _i32, _vp, _vp, _i32, _vp]
        R.ref_random_queries.argtypes = [_i32, _i32, _i32, _i32, _i32, _vp]
        _ref = R
    return _ref


def _ref_call(name, A, Q, nt, dtype):
    A, pa = _arr(A, np.float32)
    Q, pq = _arr(Q, np.int32)
    out = np.empty(len(Q), dtype=dtype)
    getattr(ref(), name)(len(A), len(Q), pa, pq, nt, out.ctypes.data)
    return out


def ref_cpu_rmq(A, Q, nt=1):
    return _ref_call("ref_cpu_rmq", A, Q, nt, np.float32)


def ref_cpu_rmq_idx(A, Q, nt=1):
    return _ref_call("ref_cpu_rmq_idx", A, Q, nt, np.int32)


def ref_hrmq_val(A, Q, nt=1):
    return _ref_call("ref_rmq_rmm_par", A, Q, nt, np.float32)


def ref_hrmq_idx(A, Q, nt=1):
    return _ref_call("ref_rmq_rmm_par_idx", A, Q, nt, np.int32)


def ref_random_queries(q, lr, n, nt, seed):
    out = np.empty((q, 2), dtype=np.int32)
    ref().ref_random_queries(q, lr, n, nt, seed, out.ctypes.data)
    return out
