"""GPU: the batched ragged form (one persistent cooperative launch) against
the CPU oracle per array, against the per-array plain path, under CUDA-graph
capture, and the autotuner."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def bits(x):
    return np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)


def small_ragged(seed, ties=False, align=1):
    """~150 arrays, lengths 1 .. 2^17 (all size buckets up to 16), starts with
    gaps and odd offsets, queries of every length class."""
    import rtxrmq_gb300 as R
    rng = np.random.default_rng(seed)
    lengths = np.concatenate([[1, 2, 3, 5, 31, 32, 33, 4095, 4096, 4097],
                              np.round(2.0 ** rng.uniform(4, 17, 140))]).astype(np.int64)
    gaps = rng.integers(0, 7, len(lengths)) * align
    padded = (lengths + align - 1) // align * align
    starts = np.cumsum(np.concatenate([[gaps[0]], padded[:-1] + gaps[1:]])).astype(np.int64)
    span = int(starts[-1] + lengths[-1] + 5)
    A = R.gen_values_int(span, 64, seed) if ties else R.gen_values_uniform(span, seed)
    qcounts = np.maximum(1, lengths // 16).astype(np.int64)
    qcounts[3] = 0  # an array without queries
    qgap = rng.integers(0, 3, len(lengths))
    qstarts = np.cumsum(np.concatenate([[0], qcounts[:-1] + qgap[1:]])).astype(np.int64)
    Q = np.zeros((int(qstarts[-1] + qcounts[-1] + 2), 2), dtype=np.int32)
    for i, (n, c, s) in enumerate(zip(lengths, qcounts, qstarts)):
        if not c:
            continue
        mode = i % 4
        if mode == 0:
            q = R.gen_queries(int(c), int(n), -1, seed + i)
        elif mode == 1:
            q = R.gen_queries_lognormal(int(c), int(n), 0.5 * np.log(n), 0.4, seed + i)
        elif mode == 2:
            q = R.gen_queries(int(c), int(n), 1, seed + i)
        else:
            q = R.gen_queries(int(c), int(n), int(min(n, 33)), seed + i)
        Q[s:s + c] = q
    return starts, lengths, qstarts, qcounts, A, Q


def expected(oracle_lib, starts, lengths, qstarts, qcounts, A, Q):
    ev = np.full(len(Q), np.nan, np.float32)
    ei = np.full(len(Q), -2, np.int32)
    for s, n, qs, qc in zip(starts, lengths, qstarts, qcounts):
        if qc:
            a = A[s:s + n]
            q = Q[qs:qs + qc]
            ev[qs:qs + qc] = oracle_lib.base_val(a, q)
            ei[qs:qs + qc] = oracle_lib.base_idx(a, q)
    return ev, ei


def owned_mask(qstarts, qcounts, total):
    m = np.zeros(total, bool)
    for s, c in zip(qstarts, qcounts):
        m[s:s + c] = True
    return m


@pytest.mark.parametrize("seed,ties,align", [(1, False, 1), (2, True, 1), (3, False, 4), (4, True, 4)])
@pytest.mark.parametrize("cfg", ["default", "small", "large", "mixed"])
def test_batch_matches_oracle(cuda, native, oracle_lib, seed, ties, align, cfg):
    import torch

    from rtxrmq_gb300.batch import RMQBatch
    starts, lengths, qstarts, qcounts, A, Q = small_ragged(seed, ties, align)
    bucket_bs = {"default": None, "small": [64] * 32, "large": [65536] * 32,
                 "mixed": [64, 1, 7, 16, 100, 256, 1000, 4096] * 4}[cfg]
    ev, ei = expected(oracle_lib, starts, lengths, qstarts, qcounts, A, Q)
    own = owned_mask(qstarts, qcounts, len(Q))
    dA = torch.from_numpy(A).to(cuda)
    dQ = torch.from_numpy(Q).to(cuda)
    with RMQBatch(starts, lengths, qstarts, qcounts, bucket_bs) as b:
        v, i = b.run(dA, dQ)
        v2, i2 = b.run_per_array(dA, dQ)
        torch.cuda.synchronize()
        v, i, v2, i2 = (x.cpu().numpy() for x in (v, i, v2, i2))
        assert b.invalid_count() == 0
    np.testing.assert_array_equal(i[own], ei[own])
    np.testing.assert_array_equal(bits(v[own]), bits(ev[own]))
    np.testing.assert_array_equal(i2[own], ei[own])
    np.testing.assert_array_equal(bits(v2[own]), bits(ev[own]))


def random_batch(seed):
    """A seeded random batch: 1-300 arrays of lengths 0 .. 2^16 placed anywhere
    in one values buffer (arrays may overlap: values are only read), query
    sets of 0-200 queries with gaps between them, queries for empty arrays
    (invalid by definition), and a random block size per size bucket."""
    import rtxrmq_gb300 as R
    rng = np.random.default_rng(500 + seed)
    k = int(rng.integers(1, 301))
    pick = rng.random(k)
    lengths = np.where(pick < 0.1, 0, np.where(pick < 0.4, rng.integers(1, 100, k),
                                               np.round(2.0 ** rng.uniform(7, 16, k)))).astype(np.int64)
    span = int(lengths.max()) + int(rng.integers(1, 200_000))
    starts = np.array([rng.integers(0, span - n + 1) for n in lengths], np.int64)
    A = (R.gen_values_int(span, 16, seed) if seed % 2 else R.gen_values_uniform(span, seed))
    qcounts = rng.integers(0, 201, k).astype(np.int64)
    qgap = rng.integers(0, 5, k)
    qstarts = np.cumsum(np.concatenate([[qgap[0]], qcounts[:-1] + qgap[1:]])).astype(np.int64)
    Q = np.zeros((int(qstarts[-1] + qcounts[-1] + 3), 2), dtype=np.int32)
    for i, (n, c, q0) in enumerate(zip(lengths, qcounts, qstarts)):
        if c and n:
            L = [-1, -3, 1, 2, 33][i % 5]
            Q[q0:q0 + c] = R.gen_queries(int(c), int(n), L if L < 0 or L <= n else -1, seed + i)
    choices = [0, 1, 3, 16, 33, 64, 100, 256, 1024, 4096, 65536]
    bucket_bs = [int(rng.choice(choices)) for _ in range(32)]
    return starts, lengths, qstarts, qcounts, A, Q, bucket_bs


@pytest.mark.parametrize("seed", range(24))
def test_batch_random(cuda, native, oracle_lib, seed):
    """random_batch: the batched launch and the per-array path against the
    oracle per array; queries of empty arrays give -1 / NaN and are counted."""
    import torch

    from rtxrmq_gb300.batch import RMQBatch
    starts, lengths, qstarts, qcounts, A, Q, bucket_bs = random_batch(seed)
    live = lengths > 0
    ev, ei = expected(oracle_lib, starts[live], lengths[live], qstarts[live], qcounts[live], A, Q)
    own = owned_mask(qstarts[live], qcounts[live], len(Q))
    dead = owned_mask(qstarts[~live], qcounts[~live], len(Q))
    dA = torch.from_numpy(A).to(cuda)
    dQ = torch.from_numpy(Q).to(cuda)
    with RMQBatch(starts, lengths, qstarts, qcounts, bucket_bs) as b:
        v, i = b.run(dA, dQ)
        torch.cuda.synchronize()
        v, i = v.cpu().numpy(), i.cpu().numpy()
        assert b.invalid_count() == int(dead.sum())
        v2, i2 = b.run_per_array(dA, dQ)
        v2, i2 = v2.cpu().numpy(), i2.cpu().numpy()
    for vv, ii in ((v, i), (v2, i2)):
        np.testing.assert_array_equal(ii[own], ei[own])
        np.testing.assert_array_equal(bits(vv[own]), bits(ev[own]))
    assert (i[dead] == -1).all() and np.isnan(v[dead]).all()


def test_batch_invalid_and_repeat(cuda, native, oracle_lib):
    """Invalid queries inside a batch give -1 / NaN and are counted; a plan
    runs repeatedly on new values without re-planning."""
    import torch

    import rtxrmq_gb300 as R
    from rtxrmq_gb300.batch import RMQBatch
    starts = np.array([0, 100, 300], np.int64)
    lengths = np.array([100, 200, 50], np.int64)
    qstarts = np.array([0, 3, 6], np.int64)
    qcounts = np.array([3, 3, 2], np.int64)
    Q = np.array([[0, 99], [5, 4], [0, 100], [0, 199], [10, 10], [-1, 0], [0, 49], [49, 50]], np.int32)
    with RMQBatch(starts, lengths, qstarts, qcounts) as b:
        for seed in range(3):
            A = R.gen_values_uniform(350, seed)
            v, i = b.run(torch.from_numpy(A).to(cuda), torch.from_numpy(Q).to(cuda))
            i = i.cpu().numpy()
            assert list(i) == [int(np.argmin(A[:100])), -1, -1, int(np.argmin(A[100:300])), 10, -1,
                               int(np.argmin(A[300:350])), -1]
        assert b.invalid_count() == 12


def test_batch_empty_arrays_and_no_queries(cuda, native, oracle_lib):
    """Empty arrays (length 0) are allowed: no structure, their queries are
    invalid; q = 0 runs are no-ops on every entry point; the per-array path
    and the autotuner accept the same plan."""
    import torch

    import rtxrmq_gb300 as R
    from rtxrmq_gb300.batch import RMQBatch, autotune
    starts = np.array([0, 64, 64, 300], np.int64)
    lengths = np.array([64, 0, 236, 0], np.int64)
    qstarts = np.array([0, 2, 4, 6], np.int64)
    qcounts = np.array([2, 2, 2, 0], np.int64)
    Q = np.array([[0, 63], [10, 20], [0, 0], [0, 5], [0, 235], [100, 200]], np.int32)
    A = R.gen_values_uniform(300, 3)
    dA, dQ = torch.from_numpy(A).to(cuda), torch.from_numpy(Q).to(cuda)
    want = [int(np.argmin(A[:64])), 10 + int(np.argmin(A[10:21])), -1, -1,
            int(np.argmin(A[64:300])), 100 + int(np.argmin(A[164:265]))]
    for cfg in (None, autotune(starts, lengths, qstarts, qcounts, dA, dQ, reps=1, cache=None)):
        with RMQBatch(starts, lengths, qstarts, qcounts, cfg) as b:
            v, i = b.run(dA, dQ)
            assert list(i.cpu().numpy()) == want
            v2, i2 = b.run_per_array(dA, dQ)
            assert list(i2.cpu().numpy()) == want
            assert b.invalid_count() == 4
    # q = 0 on the plain entry points
    with R.RMQIndex(dA, 64) as ix:
        empty = torch.empty((0, 2), dtype=torch.int32, device=cuda)
        v, i = ix.query(empty)
        assert v.numel() == 0 and i.numel() == 0
        ix.query_host(np.empty((0, 2), np.int32), np.empty(0, np.float32), np.empty(0, np.int32))
        ix.probe_gather(empty)
        torch.cuda.synchronize()
        assert ix.invalid_count() == 0


def test_batch_graph_capture(cuda, native, oracle_lib):
    """rmq_batch_run captured once in a CUDA graph and replayed on new data."""
    import torch

    import rtxrmq_gb300 as R
    from rtxrmq_gb300.batch import RMQBatch
    starts, lengths, qstarts, qcounts, A, Q = small_ragged(7, False, 4)
    own = owned_mask(qstarts, qcounts, len(Q))
    dA = torch.from_numpy(A).to(cuda)
    dQ = torch.from_numpy(Q).to(cuda)
    outv = torch.empty(len(Q), dtype=torch.float32, device=cuda)
    outi = torch.empty(len(Q), dtype=torch.int32, device=cuda)
    with RMQBatch(starts, lengths, qstarts, qcounts) as b:
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            b.run(dA, dQ, outv, outi)
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            b.run(dA, dQ, outv, outi)
        for seed in (11, 12):
            A2 = R.gen_values_int(len(A), 1000, seed)
            dA.copy_(torch.from_numpy(A2))
            g.replay()
            torch.cuda.synchronize()
            ev, ei = expected(oracle_lib, starts, lengths, qstarts, qcounts, A2, Q)
            np.testing.assert_array_equal(outi.cpu().numpy()[own], ei[own])
            np.testing.assert_array_equal(bits(outv.cpu().numpy()[own]), bits(ev[own]))


def test_autotune(cuda, native, oracle_lib, tmp_path):
    import torch

    from rtxrmq_gb300.batch import RMQBatch, autotune, bucket_of
    starts, lengths, qstarts, qcounts, A, Q = small_ragged(5, False, 4)
    dA = torch.from_numpy(A).to(cuda)
    dQ = torch.from_numpy(Q).to(cuda)
    cache = tmp_path / "tune.json"
    cfg = autotune(starts, lengths, qstarts, qcounts, dA, dQ, reps=2, queries_host=Q, cache=cache)
    present = set(int(b) for b in bucket_of(lengths))
    for bk in range(32):
        if bk in present:
            assert cfg[bk] in (64, 256, 1024, 4096, 16384, 65536)
        else:
            assert cfg[bk] == 0
    assert cache.exists()
    assert autotune(starts, lengths, qstarts, qcounts, dA, dQ, queries_host=Q, cache=cache) == cfg
    ev, ei = expected(oracle_lib, starts, lengths, qstarts, qcounts, A, Q)
    own = owned_mask(qstarts, qcounts, len(Q))
    with RMQBatch(starts, lengths, qstarts, qcounts, cfg) as b:
        assert b.info()["bucket_bs"][:32] == cfg
        v, i = b.run(dA, dQ)
        np.testing.assert_array_equal(i.cpu().numpy()[own], ei[own])


def test_batch_build_once_query_many(cuda, native, oracle_lib):
    """rmq_batch_build + rmq_batch_query: one build, several query sets of the
    plan's layout (also captured in a CUDA graph); a query without a build on
    the same values is refused."""
    import torch

    import oracle
    import rtxrmq_gb300 as R
    from rtxrmq_gb300.batch import RMQBatch
    rng = np.random.default_rng(31)
    lengths = rng.integers(1, 20000, 64).astype(np.int64)
    starts = np.concatenate([[0], np.cumsum(lengths)[:-1]]).astype(np.int64)
    qcounts = rng.integers(1, 2000, 64).astype(np.int64)
    qstarts = np.concatenate([[0], np.cumsum(qcounts)[:-1]]).astype(np.int64)
    V = rng.random(int(lengths.sum())).astype(np.float32)
    dV = torch.from_numpy(V).to(cuda)
    off = np.repeat(starts, qcounts)

    def queries(seed, lr):
        return np.concatenate([R.gen_queries(int(c), int(m), lr, seed + k)
                               for k, (m, c) in enumerate(zip(lengths, qcounts))])

    with RMQBatch(starts, lengths, qstarts, qcounts, [256] * 32) as b:
        Q0 = queries(1, -3)
        dQ = torch.from_numpy(Q0).to(cuda)
        with pytest.raises(R.RMQError, match="not built"):
            b.query(dV, dQ)
        b.build(dV)
        for seed, lr in ((1, -3), (2, -1), (3, 50)):
            Q = queries(seed, lr)
            v, i = b.query(dV, torch.from_numpy(Q).to(cuda))
            G = Q.astype(np.int64) + off[:, None]
            np.testing.assert_array_equal(i.cpu().numpy() + off, oracle.base_idx(V, G))
        other = dV.clone()
        with pytest.raises(R.RMQError, match="not built"):
            b.query(other, dQ)
        # the query half captured in a graph and replayed on new query contents
        v = torch.empty(len(Q0), dtype=torch.float32, device=cuda)
        i = torch.empty(len(Q0), dtype=torch.int32, device=cuda)
        b.query(dV, dQ, v, i)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            b.query(dV, dQ, v, i)
        Q = queries(7, -2)
        dQ.copy_(torch.from_numpy(Q).to(cuda))
        g.replay()
        torch.cuda.synchronize()
        G = Q.astype(np.int64) + off[:, None]
        np.testing.assert_array_equal(i.cpu().numpy() + off, oracle.base_idx(V, G))


def test_autotune_tiles(cuda, native, oracle_lib, tmp_path):
    """The tile autotuner picks per bucket a block size, a query-item size
    and a level-item size from its candidates; the plan reports them, the
    cache returns them, and the answers do not depend on them."""
    import torch

    from rtxrmq_gb300.batch import RMQBatch, autotune, bucket_of
    starts, lengths, qstarts, qcounts, A, Q = small_ragged(5, False, 4)
    dA = torch.from_numpy(A).to(cuda)
    dQ = torch.from_numpy(Q).to(cuda)
    cache = tmp_path / "tiles.json"
    cfg = autotune(starts, lengths, qstarts, qcounts, dA, dQ, reps=1, queries_host=Q, cache=cache,
                   tiles=True)
    present = set(int(b) for b in bucket_of(lengths))
    for bk in range(32):
        if bk in present:
            assert cfg[bk][0] in (64, 256, 1024, 4096, 16384, 65536)
            assert cfg[bk][1] in (512, 1024, 2048, 4096, 8192)
            assert cfg[bk][2] in (1024, 4096, 16384)
        else:
            assert cfg[bk] == (0, 0, 0)
    assert autotune(starts, lengths, qstarts, qcounts, dA, dQ, queries_host=Q, cache=cache,
                    tiles=True) == cfg
    ev, ei = expected(oracle_lib, starts, lengths, qstarts, qcounts, A, Q)
    own = owned_mask(qstarts, qcounts, len(Q))
    with RMQBatch(starts, lengths, qstarts, qcounts, cfg) as b:
        got = b.tiles()
        for bk in present:
            assert got[bk] == cfg[bk]
        v, i = b.run(dA, dQ)
        np.testing.assert_array_equal(i.cpu().numpy()[own], ei[own])
    # extreme schedules give the same answers
    for qc, lc in ((1, 1), (7, 3), (1 << 20, 1 << 20)):
        with RMQBatch(starts, lengths, qstarts, qcounts, [(256, qc, lc)] * 32) as b:
            v, i = b.run(dA, dQ)
            np.testing.assert_array_equal(i.cpu().numpy()[own], ei[own])
            np.testing.assert_array_equal(v.cpu().numpy()[own].view(np.uint32),
                                          ev[own].view(np.uint32))
