"""GPU: the measurement entry points of the query path.

rmq_query_stats answers like rmq_query (bit-exact, checked here against the
oracle) and counts how each query was settled. Its counts are checked
against an independent host model of the query kernel's first step: the
leftmost minimum of every unit (block, or 32-element micro-block) the query
touches, which settles the query when it lies inside [l, r]. The kernel may
only read a per-element entry or scan values for the queries that test does
not settle, so these counts are what the benchmark's algorithmic bytes are
computed from.

rmq_probe_random is checked against the same hash positions computed on
the host.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def composites(A):
    """(key << 32) | (index << 1) | negzero of every float32 element, as the
    engine orders them (smallest = leftmost minimum)."""
    b = A.view(np.uint32).astype(np.uint64)
    a = b & 0x7fffffff
    key = np.where(b & 0x80000000, (~b) & 0xffffffff, b | 0x80000000)
    key = np.where(a == 0, 0x80000000, key)
    key = np.where(a > 0x7f800000, 0xffffffff, key)
    negz = (b == 0x80000000).astype(np.uint64)
    idx = np.arange(len(A), dtype=np.uint64)
    return (key.astype(np.uint64) << np.uint64(32)) | (idx << np.uint64(1)) | negz


def unit_minima(C, width):
    pad = (-len(C)) % width
    Cp = np.concatenate([C, np.full(pad, np.iinfo(np.uint64).max, np.uint64)])
    return Cp.reshape(-1, width).min(axis=1)


def range_min(M, a, b):
    """Minimum of M[a..b] per query through a host sparse table."""
    levels = [M]
    while (1 << len(levels)) <= len(M):
        prev, h = levels[-1], 1 << (len(levels) - 1)
        levels.append(np.minimum(prev[:-h], prev[h:]))
    w = b - a + 1
    lev = np.floor(np.log2(w)).astype(np.int64)
    out = np.empty(len(a), np.uint64)
    for k in np.unique(lev):
        s = lev == k
        t = levels[k]
        out[s] = np.minimum(t[a[s]], t[b[s] + 1 - (1 << k)])
    return out


def model_first_probe(A, Q, bs, mlevels):
    """Queries settled by the superset probe, as the kernel classifies them:
    micro-block table when the query spans 2..2^mlevels-1 micro-blocks,
    block table otherwise (inside one micro-block: scanned, not probed)."""
    C = composites(A)
    l, r = Q[:, 0].astype(np.int64), Q[:, 1].astype(np.int64)
    ml, mr, lB, rB = l // 32, r // 32, l // bs, r // bs
    micro = mlevels > 0
    w = mr - ml + 1
    use_micro = micro & (ml != mr) & (np.floor(np.log2(np.maximum(w, 1))) < mlevels)
    scan = micro & (ml == mr)
    use_block = ~use_micro & ~scan
    first = 0
    if use_micro.any():
        m = range_min(unit_minima(C, 32), ml[use_micro], mr[use_micro])
        i = (m & 0xffffffff).astype(np.int64) >> 1
        first += int(((i >= l[use_micro]) & (i <= r[use_micro])).sum())
    if use_block.any():
        m = range_min(unit_minima(C, bs), lB[use_block], rB[use_block])
        i = (m & 0xffffffff).astype(np.int64) >> 1
        first += int(((i >= l[use_block]) & (i <= r[use_block])).sum())
    return first, int(scan.sum())


@pytest.mark.parametrize("bs,lr,micro", [(1 << 10, -3, True), (1 << 12, -2, True),
                                         (1 << 15, -1, True), (1 << 10, 1024, True),
                                         (128, -3, True), (1 << 12, -2, False),
                                         (1 << 10, -3, False)])
def test_query_stats_counts(cuda, native, oracle_lib, bs, lr, micro):
    import torch

    import rtxrmq_gb300 as R
    n, q = (1 << 22) + 77, 1 << 16
    A = R.gen_values_uniform(n, 31)
    Q = R.gen_queries(q, n, lr, 32)
    Q[:2] = [[3, 2], [0, n]]  # invalid
    dA = torch.from_numpy(A).to(cuda)
    dQ = torch.from_numpy(Q).to(cuda)
    with R.RMQIndex(dA, bs, micro=micro) as ix:
        v = torch.empty(q, dtype=torch.float32, device=cuda)
        i = torch.empty(q, dtype=torch.int32, device=cuda)
        st = ix.query_stats(dQ, out_val=v, out_idx=i)
        v2, i2 = ix.query(dQ)
        torch.cuda.synchronize()
        mlevels = ix.info()["micro_levels"]
    i, v = i.cpu().numpy(), v.cpu().numpy()
    np.testing.assert_array_equal(i, i2.cpu().numpy())
    np.testing.assert_array_equal(v.view(np.uint32), v2.cpu().numpy().view(np.uint32))
    ei = oracle_lib.base_idx(A, Q)
    ei[:2] = -1  # the invalid queries
    np.testing.assert_array_equal(i, ei)

    settled = sum(st[k] for k in ("first_probe", "second_probe", "full", "micro_scan",
                                  "block_edge", "warp_scan", "invalid"))
    assert settled == q, st
    assert st["invalid"] == 2
    # per-element entries: one for a second-probe query, two for the full
    # decomposition, one for a block edge
    assert st["entries"] == st["second_probe"] + 2 * st["full"] + st["block_edge"], st
    first, scans = model_first_probe(A, Q[2:], bs, mlevels)
    assert st["first_probe"] == first, (st, first)
    assert st["micro_scan"] == scans, (st, scans)
    if not micro:
        assert st["micro_scan"] == 0
    else:
        assert st["warp_scan"] == 0 and st["block_edge"] == 0


def test_probe_random_positions(cuda, native):
    import torch

    import rtxrmq_gb300 as R
    words = (1 << 20) + 3
    buf = torch.randint(-2**62, 2**62, (words,), dtype=torch.int64, device=cuda)
    Q = R.gen_queries(5000, 1 << 20, -1, 3)
    v, i = R.probe_random(buf, torch.from_numpy(Q).to(cuda))
    torch.cuda.synchronize()
    B = buf.cpu().numpy().view(np.uint64)
    v, i = v.cpu().numpy().view(np.uint32), i.cpu().numpy().view(np.uint32)
    M = (1 << 64) - 1

    def mix(x):
        x = ((x ^ (x >> 30)) * 0xbf58476d1ce4e5b9) & M
        x = ((x ^ (x >> 27)) * 0x94d049bb133111eb) & M
        return x ^ (x >> 31)

    for k in range(0, len(Q), 97):
        l, r = int(Q[k, 0]) & 0xffffffff, int(Q[k, 1]) & 0xffffffff
        h1 = mix(((k << 32) ^ l) & M)
        h2 = mix(h1 ^ r)
        e = min(int(B[(h1 * words) >> 64]), int(B[(h2 * words) >> 64]))
        assert int(v[k]) == e >> 32 and int(i[k]) == e & 0xffffffff, k
