"""rtxrmq_gb300 -- GB300-native batch range-minimum queries (RMQ).

Host-side mirror of the reference's interface for its hot path
(``rtx_rmq<T>(alg, n, bs, q, darray, dquery, args)``, src/rtx.h:24-177, with
alg 5 returning values and alg 105 returning indices; ``gpu_rmq_basic`` /
``gpu_rmq_basic_idx``, src/cuda_methods.cuh:69-169) over the C ABI of
include/rmq.h. Device buffers are torch CUDA tensors (used only as device
memory and streams); every computation runs in librmq.so.

Semantics for an inclusive query (l, r): value = min A[l..r] (the exact bits
of A[idx]) and idx = the leftmost position holding it, as the reference's
BASE oracles (src/cpu_methods.h:42-53).
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Tuple

import numpy as np

from ._native import LIB_PATH, RMQError, check, load, rmq_info_t

__all__ = [
    "RMQIndex", "RMQError", "rtx_rmq", "gpu_rmq_basic", "gpu_rmq_basic_idx", "bs_from_nb",
    "gen_values_uniform", "gen_values_normal", "gen_values_int", "gen_queries",
    "gen_queries_lognormal", "probe_random", "ALG_GPU_BASE", "ALG_GPU_RTX_BLOCKS", "ALG_GPU_BASE_IDX",
    "ALG_GPU_RTX_BLOCKS_IDX", "DEFAULT_BS", "LIB_PATH", "load",
]

# algorithm ids of src/main.cu:17-32 that this engine serves
ALG_GPU_BASE = 2
ALG_GPU_RTX_BLOCKS = 5
ALG_GPU_BASE_IDX = 102
ALG_GPU_RTX_BLOCKS_IDX = 105
DEFAULT_BS = 1 << 15  # src/tools.h:96


def _stream_handle(stream) -> Optional[int]:
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def _dptr(t) -> Optional[int]:
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return t.data_ptr()


def _check_queries(queries):
    import torch
    if queries.dtype != torch.int32:
        raise TypeError("queries must be int32 (l, r) pairs")
    if queries.dim() != 2 or queries.shape[1] != 2:
        raise ValueError("queries must have shape [q, 2]")
    return queries.shape[0]


class RMQIndex:
    """Block-decomposition index over a float32 CUDA tensor.

    Construction is the GPU replacement of RTX_blocks' geometry + BVH build
    (src/rtx.h:39-99); ``query`` replaces the timed optixLaunch
    (src/rtx.h:150-154). ``values`` must stay alive and unchanged while the
    index is used (the index refers to it, it does not copy it).
    """

    def __init__(self, values, bs: int = 0, stream=None, micro: bool = True, op: str = "min",
                 light: bool = False):
        """values: 1-D float32 or int32 CUDA tensor; op: "min" (the
        reference's semantics) or "max"; ties resolve to the leftmost index.
        light=True builds the light index (RMQ_BUILD_LIGHT: tables only, no
        per-element entries; bs a multiple of 32, >= 64)."""
        import torch
        if values.dim() != 1 or values.dtype not in (torch.float32, torch.int32):
            raise TypeError("values must be a 1-D float32 or int32 CUDA tensor")
        if op not in ("min", "max"):
            raise ValueError("op must be 'min' or 'max'")
        lib = load()
        self._values = values
        self._vdtype = values.dtype
        self._h = C.c_void_p()
        flags = ((0 if micro else 1) | (2 if op == "max" else 0) |
                 (4 if values.dtype == torch.int32 else 0) | (8 if light else 0))  # RMQ_BUILD_*
        check(lib.rmq_build_ex(_dptr(values), values.numel(), int(bs), flags,
                               _stream_handle(stream), C.byref(self._h)))

    def info(self) -> dict:
        inf = rmq_info_t()
        check(load().rmq_info(self._h, C.byref(inf)))
        return {k: getattr(inf, k) for k, _ in rmq_info_t._fields_}

    def query(self, queries, *, values: bool = True, indices: bool = True, out_val=None,
              out_idx=None, stream=None) -> Tuple:
        """Answer int32 [q, 2] queries; returns (val, idx), either may be None."""
        import torch
        q = _check_queries(queries)
        dev = queries.device
        if values and out_val is None:
            out_val = torch.empty(q, dtype=getattr(self, "_vdtype", torch.float32), device=dev)
        if indices and out_idx is None:
            out_idx = torch.empty(q, dtype=torch.int32, device=dev)
        if not values:
            out_val = None
        if not indices:
            out_idx = None
        check(load().rmq_query(self._h, _dptr(queries), q, _dptr(out_val), _dptr(out_idx),
                               _stream_handle(stream)))
        return out_val, out_idx

    def query_host(self, queries, out_val=None, out_idx=None, stream=None) -> None:
        """rmq_query_host: host-side buffers (CPU tensors or numpy arrays).
        Buffers the GPU can address (page-locked, or any memory on
        Grace-Blackwell) are read and written in place by the query kernel;
        others go through device staging. Results are valid after the stream
        is synchronised."""
        def hptr(x):
            if x is None:
                return None
            if hasattr(x, "data_ptr"):
                if not x.is_contiguous():
                    raise ValueError("expected a contiguous buffer")
                return x.data_ptr()
            if not x.flags["C_CONTIGUOUS"]:
                raise ValueError("expected a contiguous buffer")
            return x.ctypes.data
        q = len(queries)
        if tuple(queries.shape[1:]) != (2,):
            raise ValueError("queries must have shape [q, 2]")
        check(load().rmq_query_host(self._h, hptr(queries), q, hptr(out_val), hptr(out_idx),
                                    _stream_handle(stream)))

    def probe_gather(self, queries, out_val=None, out_idx=None, stream=None) -> Tuple:
        """rmq_probe_gather: the two-lookup random-access ceiling of query()
        on this index (a measurement helper; its outputs are range minima
        only for queries whose ends lie in the same or adjacent blocks)."""
        import torch
        q = _check_queries(queries)
        if out_val is None:
            out_val = torch.empty(q, dtype=getattr(self, "_vdtype", torch.float32), device=queries.device)
        if out_idx is None:
            out_idx = torch.empty(q, dtype=torch.int32, device=queries.device)
        check(load().rmq_probe_gather(self._h, _dptr(queries), q, _dptr(out_val), _dptr(out_idx),
                                      _stream_handle(stream)))
        return out_val, out_idx

    STATS_FIELDS = ("first_probe", "second_probe", "full", "micro_scan", "block_edge",
                    "warp_scan", "entries", "table_words", "scan_sectors", "invalid")

    def query_stats(self, queries, out_val=None, out_idx=None, stream=None) -> dict:
        """rmq_query_stats: the same answers as query() (into out_val /
        out_idx when given) from the counting instantiation of the query
        kernel, and how every query was settled and what it read (field
        names in STATS_FIELDS). Synchronises the stream."""
        q = _check_queries(queries)
        counts = (C.c_int64 * len(self.STATS_FIELDS))()
        check(load().rmq_query_stats(self._h, _dptr(queries), q, _dptr(out_val), _dptr(out_idx),
                                     counts, _stream_handle(stream)))
        return dict(zip(self.STATS_FIELDS, (int(x) for x in counts)))

    def save(self, path, stream=None) -> None:
        """Write the index (not the values) to ``path`` (rmq_save)."""
        check(load().rmq_save(self._h, str(path).encode(), _stream_handle(stream)))

    @classmethod
    def load(cls, values, path, stream=None) -> "RMQIndex":
        """Index for ``values`` read from ``path`` (rmq_load); the values must
        be the ones the index was built from."""
        import torch
        if values.dim() != 1 or values.dtype not in (torch.float32, torch.int32):
            raise TypeError("values must be a 1-D float32 or int32 CUDA tensor")
        self = cls.__new__(cls)
        self._values = values
        self._vdtype = values.dtype
        self._h = C.c_void_p()
        check(load().rmq_load(_dptr(values), values.numel(), str(path).encode(),
                              _stream_handle(stream), C.byref(self._h)))
        return self

    def invalid_count(self, stream=None) -> int:
        v = C.c_int64()
        check(load().rmq_invalid_count(self._h, _stream_handle(stream), C.byref(v)))
        return v.value

    @property
    def handle(self) -> int:
        return self._h.value or 0

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            check(load().rmq_free(self._h))
            self._h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def probe_random(buf, queries, out_val=None, out_idx=None, stream=None) -> Tuple:
    """rmq_probe_random: per query two random 8-byte loads from the int64
    CUDA tensor ``buf`` with the query kernel's grid, query stream and
    stores (the GPU's random-access rate, independent of any index)."""
    import torch
    q = _check_queries(queries)
    if buf.dtype != torch.int64 or buf.dim() != 1:
        raise TypeError("buf must be a 1-D int64 CUDA tensor")
    if out_val is None:
        out_val = torch.empty(q, dtype=torch.float32, device=queries.device)
    if out_idx is None:
        out_idx = torch.empty(q, dtype=torch.int32, device=queries.device)
    check(load().rmq_probe_random(_dptr(buf), buf.numel(), _dptr(queries), q, _dptr(out_val),
                                  _dptr(out_idx), _stream_handle(stream)))
    return out_val, out_idx


def bs_from_nb(n: int, nb: int) -> int:
    """--nb semantics of src/tools.h:129-132: bs = n // min(n, nb)."""
    bs = C.c_int64()
    check(load().rmq_bs_from_nb(n, nb, C.byref(bs)))
    return bs.value


def rtx_rmq(alg: int, n: int, bs: int, q: int, darray, dquery, reps: int = 1) -> np.ndarray:
    """Mirror of ``rtx_rmq<T>`` (src/rtx.h:24-177) for alg 5 / 105.

    Builds the index over ``darray[:n]`` with block size ``bs``, answers the
    first ``q`` queries of ``dquery`` ``reps`` times, and returns a host array:
    float32 values for alg 5, int32 indices for alg 105.
    """
    import torch
    if alg not in (ALG_GPU_RTX_BLOCKS, ALG_GPU_RTX_BLOCKS_IDX):
        raise RMQError(-5, f"alg {alg} is not served by rtx_rmq (use 5 or 105)")
    want_idx = alg >= 100
    with RMQIndex(darray[:n], bs) as ix:
        out = None
        for _ in range(max(1, reps)):
            v, i = ix.query(dquery[:q], values=not want_idx, indices=want_idx)
            out = i if want_idx else v
        torch.cuda.current_stream().synchronize()
        return out.cpu().numpy()


def _gpu_base(n: int, q: int, darray, dquery, want_idx: bool) -> np.ndarray:
    import torch
    _check_queries(dquery[:q])
    dev = dquery.device
    val = None if want_idx else torch.empty(q, dtype=torch.float32, device=dev)
    idx = torch.empty(q, dtype=torch.int32, device=dev) if want_idx else None
    check(load().rmq_query_scan(_dptr(darray), n, _dptr(dquery[:q]), q, _dptr(val), _dptr(idx),
                                _stream_handle(None)))
    torch.cuda.current_stream().synchronize()
    return (idx if want_idx else val).cpu().numpy()


def gpu_rmq_basic(n: int, q: int, darray, dquery) -> np.ndarray:
    """Mirror of gpu_rmq_basic (alg 2, src/cuda_methods.cuh:69-101): values."""
    return _gpu_base(n, q, darray, dquery, False)


def gpu_rmq_basic_idx(n: int, q: int, darray, dquery) -> np.ndarray:
    """Mirror of gpu_rmq_basic_idx (alg 102, src/cuda_methods.cuh:103-135): indices."""
    return _gpu_base(n, q, darray, dquery, True)


# ---- synthetic inputs (host) ----

def gen_values_uniform(n: int, seed: int) -> np.ndarray:
    out = np.empty(n, dtype=np.float32)
    check(load().rmq_gen_values_uniform(out.ctypes.data, n, seed & (2**64 - 1)))
    return out


def gen_values_normal(n: int, seed: int, mean: float = 0.0, std: float = 1.0) -> np.ndarray:
    out = np.empty(n, dtype=np.float32)
    check(load().rmq_gen_values_normal(out.ctypes.data, n, mean, std, seed & (2**64 - 1)))
    return out


def gen_values_int(n: int, value_range: int, seed: int) -> np.ndarray:
    out = np.empty(n, dtype=np.float32)
    check(load().rmq_gen_values_int(out.ctypes.data, n, value_range, seed & (2**64 - 1)))
    return out


def gen_queries(q: int, n: int, lr: int, seed: int) -> np.ndarray:
    """int32 [q, 2] queries with the reference's length modes (lr > 0, -1 .. -5)."""
    out = np.empty((q, 2), dtype=np.int32)
    check(load().rmq_gen_queries(out.ctypes.data, q, n, lr, seed & (2**64 - 1)))
    return out


def gen_queries_lognormal(q: int, n: int, mu: float, sigma: float, seed: int) -> np.ndarray:
    out = np.empty((q, 2), dtype=np.int32)
    check(load().rmq_gen_queries_lognormal(out.ctypes.data, q, n, mu, sigma, seed & (2**64 - 1)))
    return out
