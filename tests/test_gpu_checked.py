"""The range-checked build (-DRMQ_CHECKED=1), the engine's stand-in for a
memory sanitizer: every global index its kernels use is checked, and an
out-of-range one is counted (rmq_checked_violations) and skipped instead of
accessed. Every entry point is run through that build on the edge layouts
(block sizes 1 .. 2^20 around the builder's one-tile / two-phase / streamed
paths, unaligned values, invalid queries, key modes, host buffers in place
and staged, save / load, the probe, the no-allocation entry, batches with
odd offsets and empty arrays, the per-array path, the gradient scatter, and
the seeded random configurations and batches of the parity tests); the
answers must equal the oracle's and no violation may be counted."""
import json
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parent.parent

CASES = r'''
import json, sys
import numpy as np
import torch
from rtxrmq_gb300 import _native
L = _native.load(sys.argv[1])
import ctypes as C
import oracle
import rtxrmq_gb300 as R
from rtxrmq_gb300.batch import RMQBatch

dev = torch.device("cuda", 0)
ran = 0
def eq(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    if not np.array_equal(a, b):
        bad = np.nonzero(a != b)[0]
        raise SystemExit(f"{what}: {bad.size} mismatches, first at {bad[0]}")

rng = np.random.default_rng(5)
# plain index, every builder path and query path
for n in (1, 33, 300, 5000, 100_000, 300_001):
    A = rng.integers(0, 64, n).astype(np.float32)
    A[rng.integers(0, n, max(1, n // 50))] = -0.0
    Q = np.concatenate([R.gen_queries(4000, n, L_, 9)
                        for L_ in (-1, -3, 1, 2, 31, 33, 100, 700) if L_ <= n])
    if n <= 300:
        Q = np.array([(l, r) for l in range(n) for r in range(l, n)], np.int32)
    bad = np.array([[-1, 0], [0, n], [5, 4], [n, n + 1]], np.int32)
    ei, ev = oracle.base_idx(A, Q), oracle.base_val(A, Q)
    dQ = torch.from_numpy(np.concatenate([Q, bad])).to(dev)
    for off in (0, 1):  # 16-byte aligned and unaligned values
        buf = torch.zeros(n + 4, dtype=torch.float32, device=dev)
        buf[off:off + n] = torch.from_numpy(A).to(dev)
        dA = buf[off:off + n]
        for bs in (1, 7, 32, 96, 1000, 1024, 4096, 12207, 1 << 16, 1 << 18, 1 << 20):
            for micro in (True, False):
                with R.RMQIndex(dA, bs, micro=micro) as ix:
                    v, i = ix.query(dQ)
                    i = i.cpu().numpy(); v = v.cpu().numpy()
                    eq(i[:len(Q)], ei, f"idx n={n} bs={bs} micro={micro} off={off}")
                    eq(v[:len(Q)].view(np.uint32), ev.view(np.uint32), f"val n={n} bs={bs}")
                    assert (i[len(Q):] == -1).all()
                    ix.probe_gather(dQ)
                ran += 1
    # host buffers: in place (pinned) and staged
    dA = torch.from_numpy(A).to(dev)
    with R.RMQIndex(dA, 1024) as ix:
        hQ = torch.from_numpy(Q).pin_memory()
        hv, hi = torch.empty(len(Q)).pin_memory(), torch.empty(len(Q), dtype=torch.int32).pin_memory()
        ix.query_host(hQ, hv, hi); torch.cuda.synchronize(); eq(hi.numpy(), ei, "host in place")
        import os
        os.environ["RTXRMQ_HOST_STAGED"] = "1"
        hv2, hi2 = np.empty(len(Q), np.float32), np.empty(len(Q), np.int32)
        ix.query_host(Q, hv2, hi2); torch.cuda.synchronize(); eq(hi2, ei, "host staged")
        del os.environ["RTXRMQ_HOST_STAGED"]
        ix.save("/tmp/rmq_checked.ix")
    with R.RMQIndex.load(dA, "/tmp/rmq_checked.ix") as ix:
        v, i = ix.query(torch.from_numpy(Q).to(dev)); eq(i.cpu().numpy(), ei, "load")
    os.remove("/tmp/rmq_checked.ix")
    if n <= 100_000:
        nv = torch.empty(len(Q), device=dev); ni = torch.empty(len(Q), dtype=torch.int32, device=dev)
        rc = L.rmq_query_noalloc(dA.data_ptr(), n, 1024, torch.from_numpy(Q).to(dev).data_ptr(), len(Q),
                                 nv.data_ptr(), ni.data_ptr(), None)
        assert rc == 0, rc
        eq(ni.cpu().numpy(), ei, "noalloc")

# light indexes (tables only, open queries scan value lines): block sizes
# around the micro-block and block edges, unaligned values, tie-heavy
for n, bs, off in ((1000, 64, 0), (4097, 96, 1), (100_003, 1024, 2), (70_000, 65536, 0)):
    A = R.gen_values_int(n, 16, n)
    Q = R.gen_queries(20_000, n, -3, 1) if n > 2000 else np.stack(np.triu_indices(n), 1).astype(np.int32)[::7]
    ei = oracle.base_idx(A, Q)
    pad = np.zeros(off, np.float32)
    big = torch.from_numpy(np.concatenate([pad, A])).to(dev)
    with R.RMQIndex(big[off:off + n], bs, light=True) as ix:
        v, i = ix.query(torch.from_numpy(Q).to(dev))
        eq(i.cpu().numpy(), ei, f"light n={n} bs={bs} off={off}")
    ran += 1

# the no-allocation entry point on an index that fits its scratch only
# without the sub-block level (the plain-index fallback)
n = 1 << 20
A = R.gen_values_int(n, 1000, 21)
Q = R.gen_queries(50_000, n, -2, 22)
ei = oracle.base_idx(A, Q)
dA = torch.from_numpy(A).to(dev)
nv = torch.empty(len(Q), device=dev); ni = torch.empty(len(Q), dtype=torch.int32, device=dev)
rc = L.rmq_query_noalloc(dA.data_ptr(), n, 64, torch.from_numpy(Q).to(dev).data_ptr(), len(Q),
                         nv.data_ptr(), ni.data_ptr(), None)
assert rc == 0, rc
eq(ni.cpu().numpy(), ei, "noalloc plain fallback")
ran += 1

# key modes
A = rng.integers(-2**31, 2**31 - 1, 20000, dtype=np.int64).astype(np.int32)
Q = R.gen_queries(20000, len(A), -3, 4)
for op in ("min", "max"):
    f = np.argmin if op == "min" else np.argmax
    want = np.array([l + f(A[l:r + 1]) for l, r in Q], np.int32)
    for bs in (64, 1024, 1 << 15):
        with R.RMQIndex(torch.from_numpy(A).to(dev), bs, op=op) as ix:
            v, i = ix.query(torch.from_numpy(Q).to(dev)); eq(i.cpu().numpy(), want, f"int {op} bs={bs}")
        ran += 1

# batches: odd offsets, gaps, empty arrays, every block-size class
lengths = rng.integers(0, 5000, 200).astype(np.int64)
lengths[::17] = 0
starts = np.cumsum(np.concatenate([[3], lengths[:-1] + rng.integers(0, 9, 199)])).astype(np.int64)
span = int(starts[-1] + lengths[-1] + 8)
V = rng.random(span).astype(np.float32)
qc = rng.integers(0, 300, 200).astype(np.int64)
qs = np.concatenate([[0], np.cumsum(qc)[:-1]]).astype(np.int64)
Qs = []
for n_, c in zip(lengths, qc):
    if n_ == 0:
        Qs.append(np.tile(np.array([[0, 0]], np.int32), (c, 1)))
    else:
        Qs.append(R.gen_queries(int(c), int(n_), -3, 7) if c else np.zeros((0, 2), np.int32))
Qb = np.concatenate(Qs)
G = Qb.astype(np.int64) + np.repeat(starts, qc)[:, None]
nonempty = np.repeat(lengths, qc) > 0
wi = np.full(len(Qb), -1, np.int64)
wi[nonempty] = oracle.base_idx(V, G[nonempty]) - np.repeat(starts, qc)[nonempty]
dV, dQb = torch.from_numpy(V).to(dev), torch.from_numpy(Qb).to(dev)
for cfg in (None, [1] * 32, [64] * 32, [1000] * 32, [4096] * 32, [1 << 16] * 32):
    with RMQBatch(starts, lengths, qs, qc, cfg) as b:
        v, i = b.run(dV, dQb); eq(i.cpu().numpy(), wi, f"batch {cfg and cfg[0]}")
        v2, i2 = b.run_per_array(dV, dQb); eq(i2.cpu().numpy(), wi, "per-array")
        g = torch.zeros(span, device=dev)
        b.scatter_grad(i, torch.ones(len(Qb), device=dev), g)
        torch.cuda.synchronize()
        assert abs(float(g.sum()) - float(nonempty.sum())) < 0.5
    ran += 1

# the seeded random configurations of the parity tests
sys.path.insert(0, "tests")
import test_gpu_batch as TB
import test_gpu_parity as TP
for seed in range(64):
    n, bs, dtype, op, micro, off, A, Q = TP.random_case(seed)
    ei = TP.np_leftmost(A, Q, op)
    big = torch.from_numpy(np.concatenate([np.zeros(off, dtype=A.dtype), A])).to(dev)
    with R.RMQIndex(big[off:off + n], bs, micro=micro, op=op) as ix:
        v, i = ix.query(torch.from_numpy(Q).to(dev))
        eq(i.cpu().numpy(), ei, f"random case {seed}")
        eq(v.cpu().numpy().view(np.uint32), A[ei].view(np.uint32), f"random case {seed} values")
    ran += 1
for seed in range(24):
    starts, lengths, qstarts, qcounts, V, Qr, bucket_bs = TB.random_batch(seed)
    live = lengths > 0
    ev, ei = TB.expected(oracle, starts[live], lengths[live], qstarts[live], qcounts[live], V, Qr)
    own = TB.owned_mask(qstarts[live], qcounts[live], len(Qr))
    with RMQBatch(starts, lengths, qstarts, qcounts, bucket_bs) as b:
        v, i = b.run(torch.from_numpy(V).to(dev), torch.from_numpy(Qr).to(dev))
        eq(i.cpu().numpy()[own], ei[own], f"random batch {seed}")
    ran += 1
    # the same batch as a light plan (block sizes made multiples of 32, >= 64),
    # and as int32 range maximum over the same values scaled to integers
    lbs = [0 if x <= 0 else max(64, x // 32 * 32) for x in bucket_bs]
    if seed % 4 == 3:
        lbs = [1 << 18] * 32  # micro table one level per table step
    with RMQBatch(starts, lengths, qstarts, qcounts, lbs, light=True) as b:
        dVr, dQr = torch.from_numpy(V).to(dev), torch.from_numpy(Qr).to(dev)
        v, i = b.run(dVr, dQr)
        eq(i.cpu().numpy()[own], ei[own], f"random light batch {seed}")
        v, i = b.run_per_array(dVr, dQr)
        eq(i.cpu().numpy()[own], ei[own], f"random light batch {seed} per array")
    Vi = np.round(V * 1000).astype(np.int32)
    _, eim = TB.expected(oracle, starts[live], lengths[live], qstarts[live], qcounts[live],
                         -Vi.astype(np.float32), Qr)
    with RMQBatch(starts, lengths, qstarts, qcounts, lbs, op="max", dtype="int32",
                  light=bool(seed % 2)) as b:
        v, i = b.run(torch.from_numpy(Vi).to(dev), torch.from_numpy(Qr).to(dev))
        eq(i.cpu().numpy()[own], eim[own], f"random int32 max batch {seed}")
    ran += 2

cnt = C.c_int64()
rc = L.rmq_checked_violations(C.byref(cnt))
print(json.dumps({"rc": rc, "violations": cnt.value, "configurations": ran}))
'''


@pytest.fixture(scope="module")
def checked_lib():
    from rtxrmq_gb300 import build as B
    return B.build(checked=True)


def test_checked_build_has_no_violations(cuda, checked_lib, oracle_lib):
    r = subprocess.run([sys.executable, "-c", CASES, str(checked_lib)], cwd=ROOT,
                       capture_output=True, text=True, timeout=1500)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-3000:])
    res = json.loads([x for x in r.stdout.splitlines() if x.startswith("{")][-1])
    assert res["rc"] == 0, "the library is not a checked build"
    assert res["violations"] == 0
    assert res["configurations"] > 200

