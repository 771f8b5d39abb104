"""Batched ragged RMQ over the C ABI (rmq_batch_* in include/rmq.h).

Thousands of independent float32 (or int32) arrays of uneven length, each
with its own (l, r) queries, are built and answered by one persistent
cooperative kernel launch, for range minimum or maximum, with the full index
(prefix / suffix entries per element) or the light one (block and
micro-block tables only). ``run_per_array`` produces the same results
through the plain path (one build + one query launch sequence per array)
for comparison.
``autotune`` picks the block size of every size bucket (floor(log2 length))
by timing the candidates on the actual arrays and queries, and with
``tiles=True`` also the bucket's tile schedule (queries per query item,
table entries per level item); it caches the choice per GPU model, bucket
and query-length class.
"""
from __future__ import annotations

import ctypes as C
import json
import os
from pathlib import Path
from typing import Optional, Sequence

import numpy as np

from ._native import (RMQ_BATCH_BUCKETS, RMQ_BUILD_INT32, RMQ_BUILD_LIGHT, RMQ_BUILD_MAX, check,
                      load, rmq_batch_info_t, rmq_batch_tile_t)

__all__ = ["RMQBatch", "autotune", "bucket_of", "plan_flags", "DEFAULT_CACHE"]

DEFAULT_CACHE = Path(os.environ.get("RTXRMQ_AUTOTUNE_CACHE",
                                    Path.home() / ".cache" / "rtxrmq_gb300" / "autotune.json"))


def _i64(a) -> np.ndarray:
    return np.ascontiguousarray(np.asarray(a, dtype=np.int64))


def bucket_of(n) -> np.ndarray:
    n = np.asarray(n, dtype=np.int64)
    return np.where(n <= 1, 0, np.floor(np.log2(np.maximum(n, 1))).astype(np.int64))


def _stream(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    return stream if isinstance(stream, int) else stream.cuda_stream


def _dptr(t):
    if t is None:
        return None
    if not t.is_cuda or not t.is_contiguous():
        raise ValueError("expected a contiguous CUDA tensor")
    return t.data_ptr()


def _vals(t, int32: bool = False):
    """Device pointer of the flat value buffer (float32, or int32 for an
    int32 plan)."""
    import torch
    want = torch.int32 if int32 else torch.float32
    if t.dtype != want or t.dim() != 1:
        raise TypeError(f"values must be a 1-D {str(want).split('.')[-1]} CUDA tensor")
    return _dptr(t)


def plan_flags(op: str = "min", dtype="float32", light: bool = False) -> int:
    """rmq_batch_create_ex flags: range minimum or maximum, float32 or int32
    values, full or light index."""
    if op not in ("min", "max"):
        raise ValueError("op must be 'min' or 'max'")
    name = str(dtype).split(".")[-1]
    if name not in ("float32", "int32"):
        raise TypeError("dtype must be float32 or int32")
    return ((RMQ_BUILD_MAX if op == "max" else 0) | (RMQ_BUILD_INT32 if name == "int32" else 0) |
            (RMQ_BUILD_LIGHT if light else 0))


def _queries(t):
    """Device pointer of the int32 [q, 2] query tensor."""
    import torch
    if t.dtype != torch.int32 or t.dim() != 2 or t.shape[1] != 2:
        raise TypeError("queries must be an int32 CUDA tensor of shape [q, 2]")
    return _dptr(t)


def _tile_array(tiles):
    """RMQ_BATCH_BUCKETS rmq_batch_tile_t from per-bucket block sizes (ints)
    or (bs, query_chunk, level_chunk) triples; missing buckets are 0."""
    arr = (rmq_batch_tile_t * RMQ_BATCH_BUCKETS)()
    for b, t in enumerate(list(tiles)[:RMQ_BATCH_BUCKETS]):
        t = (int(t), 0, 0) if np.isscalar(t) else tuple(int(x) for x in t)
        arr[b].bs, arr[b].query_chunk, arr[b].level_chunk = t
    return arr


class RMQBatch:
    """A planned batch: array i is values[starts[i] : starts[i] + lengths[i]]
    and owns queries[qstarts[i] : qstarts[i] + qcounts[i]] (array-local
    int32 (l, r) pairs). ``bucket_bs`` maps size bucket -> block size, or
    -> (block size, queries per query item, entries per level item) as
    ``autotune(..., tiles=True)`` returns. ``op`` ("min" / "max"),
    ``dtype`` (float32 / int32 values) and ``light`` (block and micro-block
    tables only) hold for every array of the plan."""

    def __init__(self, starts: Sequence[int], lengths: Sequence[int], qstarts: Sequence[int],
                 qcounts: Sequence[int], bucket_bs: Optional[Sequence] = None, *,
                 op: str = "min", dtype="float32", light: bool = False):
        self.starts, self.lengths = _i64(starts), _i64(lengths)
        self.qstarts, self.qcounts = _i64(qstarts), _i64(qcounts)
        n = len(self.starts)
        if not (len(self.lengths) == len(self.qstarts) == len(self.qcounts) == n):
            raise ValueError("starts, lengths, qstarts, qcounts must have the same length")
        self.flags = plan_flags(op, dtype, light)
        self._int32 = bool(self.flags & RMQ_BUILD_INT32)
        tiles = None if bucket_bs is None else _tile_array(bucket_bs)
        self._h = C.c_void_p()
        check(load().rmq_batch_create_ex(n, self.starts.ctypes.data, self.lengths.ctypes.data,
                                         self.qstarts.ctypes.data, self.qcounts.ctypes.data,
                                         None if tiles is None else C.addressof(tiles),
                                         self.flags, C.byref(self._h)))

    def _out(self, queries, out_val, out_idx, values: bool, indices: bool):
        import torch
        q = queries.shape[0]
        if values and out_val is None:
            out_val = torch.empty(q, dtype=torch.int32 if self._int32 else torch.float32,
                                  device=queries.device)
        if indices and out_idx is None:
            out_idx = torch.empty(q, dtype=torch.int32, device=queries.device)
        return (out_val if values else None), (out_idx if indices else None)

    def run(self, vals, queries, out_val=None, out_idx=None, *, values=True, indices=True,
            stream=None):
        """Build + answer everything in one cooperative launch."""
        v, i = self._out(queries, out_val, out_idx, values, indices)
        check(load().rmq_batch_run(self._h, _vals(vals, self._int32), _queries(queries), _dptr(v),
                                   _dptr(i), _stream(stream)))
        return v, i

    def build(self, vals, stream=None) -> None:
        """Build every array's index (rmq_batch_build); queries then run
        with ``query`` as long as the values stay the same."""
        check(load().rmq_batch_build(self._h, _vals(vals, self._int32), _stream(stream)))

    def query(self, vals, queries, out_val=None, out_idx=None, *, values=True, indices=True,
              stream=None):
        """Answer the plan's queries from the last build on ``vals``
        (rmq_batch_query), one cooperative launch."""
        v, i = self._out(queries, out_val, out_idx, values, indices)
        check(load().rmq_batch_query(self._h, _vals(vals, self._int32), _queries(queries),
                                     _dptr(v), _dptr(i), _stream(stream)))
        return v, i

    def run_per_array(self, vals, queries, out_val=None, out_idx=None, *, values=True,
                      indices=True, stream=None):
        """Same results through the plain path, one launch sequence per array."""
        v, i = self._out(queries, out_val, out_idx, values, indices)
        check(load().rmq_batch_run_per_array(self._h, _vals(vals, self._int32), _queries(queries),
                                             _dptr(v), _dptr(i), _stream(stream)))
        return v, i

    def scatter_grad(self, idx, grad_out, grad_vals, accumulate: bool = False, stream=None):
        check(load().rmq_batch_scatter_grad(self._h, _dptr(idx), _dptr(grad_out),
                                            _dptr(grad_vals), int(bool(accumulate)),
                                            _stream(stream)))
        return grad_vals

    def info(self) -> dict:
        inf = rmq_batch_info_t()
        check(load().rmq_batch_info(self._h, C.byref(inf)))
        d = {k: getattr(inf, k) for k, _ in rmq_batch_info_t._fields_ if k != "bucket_bs"}
        d["bucket_bs"] = list(inf.bucket_bs)
        return d

    def tiles(self) -> list:
        """(block size, queries per query item, entries per level item) per
        size bucket, defaults filled in (block size 0: the default rule)."""
        arr = (rmq_batch_tile_t * RMQ_BATCH_BUCKETS)()
        check(load().rmq_batch_tiles(self._h, C.addressof(arr)))
        return [(t.bs, t.query_chunk, t.level_chunk) for t in arr]

    def invalid_count(self, stream=None) -> int:
        v = C.c_int64()
        check(load().rmq_batch_invalid_count(self._h, _stream(stream), C.byref(v)))
        return v.value

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            check(load().rmq_batch_free(self._h))
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


def _cache_keys(lengths, qstarts, qcounts, queries_host) -> dict:
    """bucket -> key 'b<bucket>_q<log2 mean query length>'."""
    keys = {}
    bk = bucket_of(lengths)
    for b in np.unique(bk):
        members = np.nonzero(bk == b)[0]
        if queries_host is None:
            qcls = "na"
        else:
            tot, cnt = 0.0, 0
            for i in members[:64]:
                s, c = int(qstarts[i]), int(min(qcounts[i], 4096))
                if c:
                    q = queries_host[s:s + c]
                    tot += float((q[:, 1] - q[:, 0] + 1).sum())
                    cnt += c
            qcls = str(int(round(np.log2(max(tot / max(cnt, 1), 1.0)))))
        keys[int(b)] = f"b{int(b)}_q{qcls}"
    return keys


def autotune(starts, lengths, qstarts, qcounts, vals, queries, *, reps: int = 3,
             queries_host: Optional[np.ndarray] = None, cache: Optional[Path] = DEFAULT_CACHE,
             stream=None, tiles: bool = False, op: str = "min", light: bool = False) -> list:
    """Per-bucket block sizes for this batch (RMQ_BATCH_BUCKETS entries), or
    with ``tiles=True`` per-bucket (block size, queries per query item,
    entries per level item) triples (rmq_batch_autotune_ex), for plans with
    ``op`` and ``light`` (and the dtype of ``vals``).

    Cached results (per GPU model and bucket/query-length key) are reused;
    missing buckets are timed on the real data."""
    import torch
    starts, lengths = _i64(starts), _i64(lengths)
    qstarts, qcounts = _i64(qstarts), _i64(qcounts)
    flags = plan_flags(op, vals.dtype, light)
    if flags != plan_flags("min", "float32", False) and not tiles:
        raise ValueError("op, int32 values and light plans are tuned with tiles=True")
    dev = torch.cuda.get_device_name()
    suffix = ("_tiles" if tiles else "") + (f"_f{flags}" if flags else "")
    keys = {b: k + suffix for b, k in _cache_keys(lengths, qstarts, qcounts, queries_host).items()}
    table = {}
    if cache is not None and Path(cache).exists():
        try:
            table = json.loads(Path(cache).read_text()).get(dev, {})
        except (OSError, ValueError):
            table = {}
    empty = (0, 0, 0) if tiles else 0
    out = [empty] * RMQ_BATCH_BUCKETS
    missing = [b for b, k in keys.items() if k not in table]
    for b, k in keys.items():
        if k in table:
            out[b] = tuple(table[k]) if tiles else int(table[k])
    if missing:
        sel = np.nonzero(np.isin(bucket_of(lengths), missing))[0]
        qn = int(queries.shape[0])
        sv = torch.empty(qn, dtype=vals.dtype, device=queries.device)
        si = torch.empty(qn, dtype=torch.int32, device=queries.device)
        s_, l_, qs_, qc_ = (np.ascontiguousarray(x[sel]) for x in (starts, lengths, qstarts, qcounts))
        args = (len(sel), s_.ctypes.data, l_.ctypes.data, qs_.ctypes.data, qc_.ctypes.data,
                _dptr(vals), _dptr(queries), _dptr(sv), _dptr(si), int(reps), _stream(stream))
        if tiles:
            res = (rmq_batch_tile_t * RMQ_BATCH_BUCKETS)()
            check(load().rmq_batch_autotune_ex(*args, flags, C.addressof(res)))
            got = [(t.bs, t.query_chunk, t.level_chunk) for t in res]
        else:
            res = np.zeros(RMQ_BATCH_BUCKETS, dtype=np.int32)
            check(load().rmq_batch_autotune(*args, res.ctypes.data))
            got = [int(x) for x in res]
        for b in missing:
            out[b] = got[b]
            table[keys[b]] = list(got[b]) if tiles else got[b]
        if cache is not None:
            try:
                Path(cache).parent.mkdir(parents=True, exist_ok=True)
                full = json.loads(Path(cache).read_text()) if Path(cache).exists() else {}
                full[dev] = table
                Path(cache).write_text(json.dumps(full, indent=1, sort_keys=True))
            except (OSError, ValueError):
                pass
    return out
