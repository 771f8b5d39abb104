"""GPU parity at the benchmark sizes.

Plain RMQ at n = 1e8, q = 2^26 for every length mode, the tie-heavy
configuration (n = 2^27 integers in [0,256), q = 2^26, fixed lengths
1 .. 2^22) and the batched ragged configuration (4096 arrays, 2^26 queries):
  * every answer is checked exactly against HRMQ, the reference's CPU
    comparator restated in the oracle (hrmq_port.c, pinned to the
    reference's own HRMQ outputs), in its leftmost-tie mode, run on all host
    cores (brute force over 2^26 long ranges is out of reach on the CPU);
  * every answer is checked for size-independent properties: l <= idx <= r
    and the value is bit-identical to A[idx];
  * a random sample is also checked against the oracle's restatement of the
    reference's block decomposition, and for short lengths against BASE.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def check_properties(A, Q, v, i):
    l, r = Q[:, 0], Q[:, 1]
    assert (i >= l).all() and (i <= r).all(), "index outside its range"
    np.testing.assert_array_equal(A[i].view(np.uint32), v.view(np.uint32))


def sampled_exact(oracle_lib, A, Q, v, i, m, seed, base=False):
    rng = np.random.default_rng(seed)
    s = rng.integers(0, len(Q), m)
    if base:
        ev, ei = oracle_lib.base_val(A, Q[s]), oracle_lib.base_idx(A, Q[s])
    else:
        ev, ei = oracle_lib.Blocks(A, 1 << 12).query(Q[s])
    np.testing.assert_array_equal(i[s], ei)
    np.testing.assert_array_equal(v[s].view(np.uint32), ev.view(np.uint32))


@pytest.fixture(scope="module")
def plain_data(cuda, native):
    import torch

    import rtxrmq_gb300 as R
    A = R.gen_values_uniform(10**8, 1321)
    return A, torch.from_numpy(A).to(cuda)


@pytest.fixture(scope="module")
def plain_hrmq(plain_data, oracle_lib):
    h = oracle_lib.HRMQ(plain_data[0], strict=True)
    yield h
    h.close()


def hrmq_exact(h, Q, v, i):
    """Every answer against HRMQ (leftmost ties)."""
    hv, hi = h.query(Q)
    bad = np.nonzero(hi != i)[0]
    assert bad.size == 0, f"{bad.size} index mismatches vs HRMQ; first q={bad[0]} (l,r)={tuple(Q[bad[0]])}"
    np.testing.assert_array_equal(v.view(np.uint32), hv.view(np.uint32))


# the block sizes the benchmark's sweep settles on per mode, and 4096
@pytest.mark.parametrize("lr,bs", [(-1, 4096), (-1, 1 << 16), (-2, 4096), (-2, 1 << 14),
                                   (-3, 4096), (-3, 1024), (1024, 4096), (1024, 1024)])
def test_plain_n1e8_q2e26(cuda, native, oracle_lib, plain_data, plain_hrmq, lr, bs):
    import torch

    import rtxrmq_gb300 as R
    A, dA = plain_data
    Q = R.gen_queries(1 << 26, len(A), lr, 1322)
    dQ = torch.from_numpy(Q).to(cuda)
    with R.RMQIndex(dA, bs) as ix:
        v, i = ix.query(dQ)
        torch.cuda.synchronize()
        assert ix.invalid_count() == 0
    v, i = v.cpu().numpy(), i.cpu().numpy()
    check_properties(A, Q, v, i)
    hrmq_exact(plain_hrmq, Q, v, i)
    sampled_exact(oracle_lib, A, Q, v, i, 1 << 14, 7)
    if lr in (-3, 1024):
        sampled_exact(oracle_lib, A, Q, v, i, 1 << 18, 8, base=True)


@pytest.mark.parametrize("length", [1, 32, 1 << 10, 1 << 16, 1 << 22])
def test_tie_heavy_n2e27_q2e26(cuda, native, oracle_lib, length):
    import torch

    import rtxrmq_gb300 as R
    n = 1 << 27
    A = R.gen_values_int(n, 256, 1321)
    Q = R.gen_queries(1 << 26, n, length, 1323)
    dA = torch.from_numpy(A).to(cuda)
    dQ = torch.from_numpy(Q).to(cuda)
    with R.RMQIndex(dA, 4096) as ix:
        v, i = ix.query(dQ)
        torch.cuda.synchronize()
    v, i = v.cpu().numpy(), i.cpu().numpy()
    check_properties(A, Q, v, i)
    h = oracle_lib.HRMQ(A, strict=True)
    hrmq_exact(h, Q, v, i)
    h.close()
    sampled_exact(oracle_lib, A, Q, v, i, 1 << 13, 9)
    if length <= 1 << 10:
        sampled_exact(oracle_lib, A, Q, v, i, 1 << 16, 10, base=True)
    del dA, dQ
    torch.cuda.empty_cache()


@pytest.mark.parametrize("bucket_bs,light", [(None, False), ([256] * 32, False),
                                             ([64] * 17 + [256] * 15, False), (None, True)])
def test_batched_ragged_full(cuda, native, oracle_lib, bucket_bs, light):
    """Batched ragged configuration at full size (4096 arrays, lengths
    round(2^U) with U ~ U[8,22], 2^26 queries), full and light index: every
    answer's properties, every answer exactly against HRMQ and a sample
    against BASE, both on the shared value buffer (a query (l, r) of the
    array at offset o is the global query (o+l, o+r))."""
    import torch

    from rtxrmq_gb300 import workloads as W
    from rtxrmq_gb300.batch import RMQBatch
    w = W.ragged()
    dV = torch.from_numpy(w.values).to(cuda)
    dQ = torch.from_numpy(w.queries).to(cuda)
    with RMQBatch(w.starts, w.lengths, w.qstarts, w.qcounts, bucket_bs, light=light) as b:
        v, i = b.run(dV, dQ)
        torch.cuda.synchronize()
        assert b.invalid_count() == 0
    v, i = v.cpu().numpy(), i.cpu().numpy().astype(np.int64)
    off = np.repeat(w.starts, w.qcounts)
    G = w.queries.astype(np.int64) + off[:, None]
    gi = i + off
    assert (gi >= G[:, 0]).all() and (gi <= G[:, 1]).all(), "index outside its range"
    np.testing.assert_array_equal(w.values[gi].view(np.uint32), v.view(np.uint32))
    # every answer against HRMQ over the shared value buffer
    h = oracle_lib.HRMQ(w.values, strict=True)
    hv, hi = h.query(G.astype(np.int32))
    h.close()
    np.testing.assert_array_equal(gi, hi)
    np.testing.assert_array_equal(v.view(np.uint32), hv.view(np.uint32))
    s = np.random.default_rng(12).integers(0, len(G), 1 << 14)
    ev, ei = oracle_lib.base_val(w.values, G[s]), oracle_lib.base_idx(w.values, G[s])
    np.testing.assert_array_equal(gi[s], ei)
    np.testing.assert_array_equal(v[s].view(np.uint32), ev.view(np.uint32))
    del dV, dQ
    torch.cuda.empty_cache()


@pytest.mark.parametrize("micro", [True, False])
def test_maximum_size_n2e31(cuda, native, oracle_lib, micro):
    """The largest supported array, n = 2^31 - 1 (indices are int32): build
    with and without the sub-block level, 2^22 queries of every length mode
    plus queries touching the last elements; every answer's properties,
    short ranges exactly against BASE, long ranges near the end against the
    GPU brute force (alg 2 / 102)."""
    import torch

    import rtxrmq_gb300 as R
    n = 2**31 - 1
    A = R.gen_values_uniform(n, 77)
    dA = torch.from_numpy(A).to(cuda)
    parts = [R.gen_queries(1 << 20, n, lr, 40 + k) for k, lr in enumerate((-1, -2, -3, 32))]
    tail = np.array([[n - 1, n - 1], [n - 2, n - 1], [n - 1000, n - 1], [0, n - 1],
                     [n - (1 << 20), n - 1], [n - 40, n - 33]], np.int32)
    Q = np.concatenate(parts + [tail])
    dQ = torch.from_numpy(Q).to(cuda)
    with R.RMQIndex(dA, 0, micro=micro) as ix:  # default bs = 2^15
        assert ix.info()["n"] == n
        v, i = ix.query(dQ)
        torch.cuda.synchronize()
        assert ix.invalid_count() == 0
    v, i = v.cpu().numpy(), i.cpu().numpy()
    check_properties(A, Q, v, i)
    short = np.nonzero(Q[:, 1] - Q[:, 0] < 4096)[0]
    sel = short[np.random.default_rng(3).integers(0, len(short), 1 << 16)]
    np.testing.assert_array_equal(i[sel], oracle_lib.base_idx(A, Q[sel]))
    # ranges at the end of the array against the GPU brute force (one thread
    # per query), the whole array against numpy's first-occurrence argmin
    first = len(Q) - len(tail)
    sub = np.array([first + k for k in range(len(tail)) if k != 3])
    bi = R.gpu_rmq_basic_idx(n, len(sub), dA, torch.from_numpy(Q[sub]).to(cuda))
    np.testing.assert_array_equal(i[sub], bi)
    assert i[first + 3] == int(np.argmin(A))
    del dA, dQ
    torch.cuda.empty_cache()
