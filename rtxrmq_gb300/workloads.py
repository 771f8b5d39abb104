"""Synthetic workloads with the shapes of the benchmark configurations.

plain(n, q, lr, seed)        -- one float32 array U[0,1) and q queries with the
                                reference's length modes (src/rand.cuh:179-201).
ragged(...)                  -- many arrays of length round(2^U), U ~ U[umin, umax],
                                queries proportional to length with lengths
                                lognormal(qmu * ln len_i, qsigma).
differentiable_rows(...)     -- rows of N(0,1) values, lengths uniform in
                                [lmin, lmax], a fixed number of queries per row
                                with lengths lognormal(qmu * ln len, qsigma).
All host-side, deterministic in the seed.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import gen_queries, gen_queries_lognormal, gen_values_normal, gen_values_uniform


@dataclass
class Ragged:
    starts: np.ndarray     # int64 [narrays]
    lengths: np.ndarray    # int64 [narrays]
    qstarts: np.ndarray    # int64 [narrays]
    qcounts: np.ndarray    # int64 [narrays]
    values: np.ndarray     # float32 [span]
    queries: np.ndarray    # int32 [total_q, 2], array-local

    @property
    def span(self) -> int:
        return int(len(self.values))

    @property
    def total_q(self) -> int:
        return int(len(self.queries))


def plain(n: int, q: int, lr: int, seed: int = 1321):
    return gen_values_uniform(n, seed), gen_queries(q, n, lr, seed + 1)


def _layout(lengths: np.ndarray, align: int):
    padded = (lengths + align - 1) // align * align
    starts = np.concatenate([[0], np.cumsum(padded)[:-1]]).astype(np.int64)
    return starts, int(starts[-1] + lengths[-1])


def _queries_for(lengths, qcounts, qmu, qsigma, seed):
    qstarts = np.concatenate([[0], np.cumsum(qcounts)[:-1]]).astype(np.int64)
    Q = np.empty((int(qcounts.sum()), 2), dtype=np.int32)
    for i, (n, c, s) in enumerate(zip(lengths, qcounts, qstarts)):
        if c:
            Q[s:s + c] = gen_queries_lognormal(int(c), int(n), qmu * float(np.log(n)), qsigma,
                                               seed * 7919 + i)
    return qstarts, Q


def ragged(narrays: int = 4096, umin: float = 8.0, umax: float = 22.0, total_q: int = 1 << 26,
           qmu: float = 0.5, qsigma: float = 0.4, seed: int = 1321, align: int = 4) -> Ragged:
    """Batched ragged configuration: 4096 arrays, lengths round(2^U) with
    U ~ U[8, 22], 2^26 queries in proportion to length, query lengths
    lognormal(0.5 ln len_i, 0.4), values U[0,1)."""
    rng = np.random.default_rng(seed)
    lengths = np.round(2.0 ** rng.uniform(umin, umax, narrays)).astype(np.int64)
    lengths = np.maximum(lengths, 1)
    share = lengths / lengths.sum()
    qcounts = np.floor(share * total_q).astype(np.int64)
    rest = total_q - int(qcounts.sum())
    if rest > 0:
        qcounts[np.argsort(-(share * total_q - qcounts))[:rest]] += 1
    starts, span = _layout(lengths, align)
    values = gen_values_uniform(span, seed + 11)
    qstarts, Q = _queries_for(lengths, qcounts, qmu, qsigma, seed + 13)
    return Ragged(starts, lengths, qstarts, qcounts, values, Q)


def differentiable_rows(nrows: int = 256, lmin: int = 1 << 14, lmax: int = 1 << 20,
                        q_per_row: int = 1 << 16, qmu: float = 0.4, qsigma: float = 0.5,
                        seed: int = 1321) -> Ragged:
    """Differentiable configuration: rows of N(0,1) values stored back to
    back, lengths uniform in [2^14, 2^20], 2^16 ranges per row with lengths
    lognormal(0.4 ln len, 0.5)."""
    rng = np.random.default_rng(seed)
    lengths = rng.integers(lmin, lmax + 1, nrows).astype(np.int64)
    starts = np.concatenate([[0], np.cumsum(lengths)[:-1]]).astype(np.int64)
    values = gen_values_normal(int(lengths.sum()), seed + 17)
    qcounts = np.full(nrows, q_per_row, dtype=np.int64)
    qstarts, Q = _queries_for(lengths, qcounts, qmu, qsigma, seed + 19)
    return Ragged(starts, lengths, qstarts, qcounts, values, Q)
