"""Speed of the HRMQ restatement (hrmq_port.c) against the reference's own
HRMQ -- TEST INFRASTRUCTURE, run where the reference tree is present.

The GPU host cannot build the reference (its sources are not there), so the
benchmark's CPU baseline is the restatement. This script measures how its
query rate compares with the real thing: the reference's rmq_rmm_par_idx
(src/cpu_methods.h:121-159 over hrmq/RMQRMM64.cpp, compiled unmodified into
oracle/_ref/libref.so by oracle/Makefile) and the restatement answer the
same queries over the same array with the same thread count, and each
query loop alone is timed (construction apart), as src/cpu_methods.h:144-154
does. The reference prints its own rate; it is read from its output.

    RTXRMQ_REFERENCE=<reference tree> python oracle/calibrate_hrmq.py [--n N] [--q Q] [--nt T]

Inputs: bench.py's numpy generators (values uniform in [0, 1), the
reference's length modes), so the arrays and queries are the benchmark's.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import re
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402

CHILD = r'''
import sys, numpy as np, oracle
A = np.load(sys.argv[1]); Q = np.load(sys.argv[2]); nt = int(sys.argv[3])
oracle.ref_hrmq_idx(A, Q, nt)
'''


def bench_module():
    spec = importlib.util.spec_from_file_location("bench", ROOT / "bench.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def reference_rate(A, Q, nt, tmp: Path):
    """Queries/s and construction seconds of the reference's rmq_rmm_par_idx,
    from its own printed timings (query loop only, as it reports them)."""
    np.save(tmp / "A.npy", A)
    np.save(tmp / "Q.npy", Q)
    r = subprocess.run([sys.executable, "-c", CHILD, str(tmp / "A.npy"), str(tmp / "Q.npy"), str(nt)],
                       cwd=ROOT, capture_output=True, text=True, timeout=3600)
    if r.returncode != 0:
        raise RuntimeError(r.stderr[-2000:])
    m = re.search(r"\[([0-9.]+) RMQs/sec", r.stdout)
    b = re.search(r"Creating MinMaxTree\.*done: ([0-9.]+) ms", r.stdout)
    if not m:
        raise RuntimeError("no rate in the reference's output:\n" + r.stdout[-2000:])
    return float(m.group(1)), (float(b.group(1)) / 1e3 if b else None)


def port_rate(A, Q, nt, strict):
    t = time.perf_counter()
    h = oracle.HRMQ(A, strict=strict, nt=nt)
    build_s = time.perf_counter() - t
    h.query(Q[:4096], nt)  # warm
    t = time.perf_counter()
    h.query(Q, nt)
    dt = time.perf_counter() - t
    h.close()
    return len(Q) / dt, build_s


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=10**8)
    ap.add_argument("--q", type=int, default=1 << 22)
    ap.add_argument("--nt", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--modes", default="-1,-2,-3,1024")
    args = ap.parse_args()
    oracle.build(with_ref=True)
    bench = bench_module()
    A = bench.np_values_uniform(args.n, bench.SEED)
    tmp = Path(os.environ.get("TMPDIR", "/tmp")) / "rtxrmq_calibrate"
    tmp.mkdir(parents=True, exist_ok=True)
    for lr in (int(x) for x in args.modes.split(",")):
        Q = bench.np_queries(args.q, args.n, lr, bench.query_seed(0, lr))
        ref_qs, ref_build = reference_rate(A, Q, args.nt, tmp)
        port_qs, port_build = port_rate(A, Q, args.nt, strict=True)
        port_r_qs, _ = port_rate(A, Q, args.nt, strict=False)
        print(json.dumps({"lr": lr, "n": args.n, "q": args.q, "nt": args.nt,
                          "reference_hrmq_rmq_s": ref_qs, "reference_build_s": ref_build,
                          "port_leftmost_rmq_s": port_qs, "port_rightmost_rmq_s": port_r_qs,
                          "port_build_s": port_build, "port_over_reference": port_qs / ref_qs}),
              flush=True)
    for f in ("A.npy", "Q.npy"):
        (tmp / f).unlink(missing_ok=True)


if __name__ == "__main__":
    main()
