"""Generate the golden vectors under tests/golden/ by running the reference's
own CPU RMQ code (cpu_rmq, cpu_rmq_idx, rmq_rmm_par, rmq_rmm_par_idx from
src/cpu_methods.h, and random_queries_par_cpu from src/rand.cuh), compiled
unmodified from the reference tree into oracle/_ref/libref.so by
oracle/Makefile.

Run from the repository root where the reference tree exists:
    make -C oracle all ref && python tests/golden/make_golden.py
Each case is one compressed .npz holding the inputs (A, Q) and the
reference's outputs:
    base_val, base_idx   -- alg 0 / 100 (BASE, leftmost)
    hrmq_val, hrmq_idx   -- alg 1 / 101 (HRMQ; indices rightmost on ties)
    hrmq_rev_idx         -- HRMQ on the reversed array with (n-1-r, n-1-l),
                            mapped back: leftmost on ties
HRMQ outputs are stored only where the reference's int reinterpretation of
the floats (src/main.cu:118-123) is order preserving (no negative values).
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
import rtxrmq_gb300 as R  # noqa: E402


def reversed_hrmq_idx(A, Q):
    n = len(A)
    Ar = np.ascontiguousarray(A[::-1])
    Qr = np.stack([n - 1 - Q[:, 1], n - 1 - Q[:, 0]], axis=1).astype(np.int32)
    return (n - 1 - oracle.ref_hrmq_idx(Ar, Qr, 1)).astype(np.int32)


def case(name, A, Q, hrmq=True, note=""):
    A = np.ascontiguousarray(A, dtype=np.float32)
    Q = np.ascontiguousarray(Q, dtype=np.int32)
    out = dict(A=A, Q=Q, base_val=oracle.ref_cpu_rmq(A, Q, 1), base_idx=oracle.ref_cpu_rmq_idx(A, Q, 1),
               note=np.array(note))
    if hrmq:
        out.update(hrmq_val=oracle.ref_hrmq_val(A, Q, 1), hrmq_idx=oracle.ref_hrmq_idx(A, Q, 1),
                   hrmq_rev_idx=reversed_hrmq_idx(A, Q))
    np.savez_compressed(HERE / f"{name}.npz", **out)
    print(name, len(A), len(Q), sorted(out))


def all_pairs(n):
    l, r = np.triu_indices(n)
    return np.stack([l, r], axis=1).astype(np.int32)


def main():
    if not oracle.ref_available():
        raise SystemExit("oracle/_ref/libref.so missing: run `make -C oracle ref` first")
    # 1. config-1 shape, scaled down: uniform values, small-range (lr=-3) and
    #    uniform-length (lr=-1) queries from this project's generator
    n = 20000
    A = R.gen_values_uniform(n, 1321)
    case("uniform_lr3", A, R.gen_queries(4096, n, -3, 1321 + 7), note="n=20000 U[0,1) lr=-3")
    case("uniform_lr1", A, R.gen_queries(4096, n, -1, 1321 + 8), note="n=20000 U[0,1) lr=-1")
    # 2. queries drawn by the reference's own generator (nt=1)
    n = 10000
    A = R.gen_values_uniform(n, 77)
    for lr in (-1, -2, -3, 100):
        case(f"refgen_lr{abs(lr)}", A, oracle.ref_random_queries(2048, lr, n, 1, 1321),
             note=f"n=10000 queries from random_queries_par_cpu(lr={lr}, nt=1, seed=1321)")
    # 3. tie-heavy: integers in [0, 16)
    n = 4096
    A = R.gen_values_int(n, 16, 5)
    Q = np.concatenate([R.gen_queries(1024, n, L, 40 + L) for L in (1, 32, 256, 1000)]
                       + [R.gen_queries(1024, n, -1, 99)])
    case("ties_int16", A, Q, note="n=4096 integers in [0,16); fixed len 1/32/256/1000 and lr=-1")
    # 4. exhaustive: every (l, r) over a small array with many ties
    A = R.gen_values_int(97, 5, 11)
    case("exhaustive_97", A, all_pairs(97), note="n=97 integers in [0,5), all 4753 ranges")
    # 5. special values (BASE only: HRMQ's int view is not order preserving)
    rng = np.random.default_rng(3)
    A = rng.standard_normal(2000).astype(np.float32)
    A[rng.integers(0, 2000, 200)] = 0.0
    A[rng.integers(0, 2000, 200)] = -0.0
    A[rng.integers(0, 2000, 20)] = np.inf
    A[rng.integers(0, 2000, 20)] = -np.inf
    A[rng.integers(0, 2000, 20)] = np.float32(1e-40)  # subnormal
    Q = np.concatenate([R.gen_queries(1024, 2000, L, 50 + L) for L in (1, 2, 17, 300)]
                       + [R.gen_queries(1024, 2000, -1, 51)])
    case("special_values", A, Q, hrmq=False,
         note="n=2000 N(0,1) with +-0, +-inf and subnormals; BASE only")


if __name__ == "__main__":
    main()
