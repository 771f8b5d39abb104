"""GPU: the batched form's light index (block and micro-block tables only)
and key modes (int32 values, range maximum), through the C ABI, against the
oracle per array: the one cooperative launch, the per-array plain path, the
build / query halves and CUDA-graph capture.

int32 values and range maximum reuse the float-minimum oracle: the int32
values here are small integers, exact as float32, and the leftmost argmax
of x is the leftmost argmin of -x (negation is exact)."""
import numpy as np
import pytest

from test_gpu_batch import bits, expected, owned_mask, random_batch, small_ragged

pytestmark = pytest.mark.gpu


def light_bs(cfg):
    """Block sizes valid for a light plan (multiples of 32, >= 64; 0 = default)."""
    if cfg is None:
        return None
    return [0 if x <= 0 else max(64, x // 32 * 32) for x in cfg]


def run_all(cuda, b, A, Q):
    """(values, indices) of run, run_per_array and build + query."""
    import torch
    dA = torch.from_numpy(A).to(cuda)
    dQ = torch.from_numpy(Q).to(cuda)
    outs = [b.run(dA, dQ), b.run_per_array(dA, dQ)]
    b.build(dA)
    outs.append(b.query(dA, dQ))
    torch.cuda.synchronize()
    return [(v.cpu().numpy(), i.cpu().numpy()) for v, i in outs]


@pytest.mark.parametrize("seed,ties,align", [(1, False, 1), (2, True, 1), (3, False, 4), (4, True, 4)])
@pytest.mark.parametrize("cfg", ["default", "small", "large", "huge", "mixed"])
def test_batch_light_matches_oracle(cuda, native, oracle_lib, seed, ties, align, cfg):
    """Light plans at every block-size class: tiles with block minima (bs/32
    dividing the tile), tiles without (bs 96, 160, 320), and blocks above
    65536 whose micro table is built one level per table step ("huge")."""
    from rtxrmq_gb300.batch import RMQBatch
    starts, lengths, qstarts, qcounts, A, Q = small_ragged(seed, ties, align)
    bucket_bs = {"default": None, "small": [64] * 32, "large": [65536] * 32,
                 "huge": [1 << 18] * 32,
                 "mixed": [64, 96, 128, 160, 320, 1024, 2048, 4096] * 4}[cfg]
    ev, ei = expected(oracle_lib, starts, lengths, qstarts, qcounts, A, Q)
    own = owned_mask(qstarts, qcounts, len(Q))
    with RMQBatch(starts, lengths, qstarts, qcounts, bucket_bs, light=True) as b:
        assert b.info()["flags"] == 8
        outs = run_all(cuda, b, A, Q)
        assert b.invalid_count() == 0
    for v, i in outs:
        np.testing.assert_array_equal(i[own], ei[own])
        np.testing.assert_array_equal(bits(v[own]), bits(ev[own]))


@pytest.mark.parametrize("seed", range(16))
def test_batch_light_random(cuda, native, oracle_lib, seed):
    """random_batch (lengths 0 .. 2^16 anywhere in the buffer, overlapping
    arrays, empty arrays with queries, a random block size per bucket) on a
    light plan, against the oracle; empty arrays' queries are invalid."""
    import torch

    from rtxrmq_gb300.batch import RMQBatch
    starts, lengths, qstarts, qcounts, A, Q, bucket_bs = random_batch(seed)
    live = lengths > 0
    ev, ei = expected(oracle_lib, starts[live], lengths[live], qstarts[live], qcounts[live], A, Q)
    own = owned_mask(qstarts[live], qcounts[live], len(Q))
    dead = owned_mask(qstarts[~live], qcounts[~live], len(Q))
    with RMQBatch(starts, lengths, qstarts, qcounts, light_bs(bucket_bs), light=True) as b:
        v, i = b.run(torch.from_numpy(A).to(cuda), torch.from_numpy(Q).to(cuda))
        torch.cuda.synchronize()
        v, i = v.cpu().numpy(), i.cpu().numpy()
        assert b.invalid_count() == int(dead.sum())
    np.testing.assert_array_equal(i[own], ei[own])
    np.testing.assert_array_equal(bits(v[own]), bits(ev[own]))
    assert (i[dead] == -1).all() and np.isnan(v[dead]).all()


@pytest.mark.parametrize("bs", [None, 64, 128])
def test_batch_light_short_arrays(cuda, native, oracle_lib, bs):
    """Every (l, r) of arrays of 1 .. 70 elements (one block of at least 64,
    one or two micro-blocks, ragged tails), tie-heavy, at odd offsets."""
    import rtxrmq_gb300 as R
    from rtxrmq_gb300.batch import RMQBatch
    lengths = np.arange(1, 71, dtype=np.int64)
    starts = np.cumsum(np.concatenate([[3], lengths[:-1] + 1])).astype(np.int64)
    A = R.gen_values_int(int(starts[-1] + lengths[-1] + 1), 5, 17)
    qs = [np.stack(np.triu_indices(int(n)), axis=1).astype(np.int32) for n in lengths]
    qcounts = np.array([len(q) for q in qs], np.int64)
    qstarts = np.concatenate([[0], np.cumsum(qcounts)[:-1]]).astype(np.int64)
    Q = np.concatenate(qs)
    ev, ei = expected(oracle_lib, starts, lengths, qstarts, qcounts, A, Q)
    with RMQBatch(starts, lengths, qstarts, qcounts, None if bs is None else [bs] * 32,
                  light=True) as b:
        outs = run_all(cuda, b, A, Q)
    for v, i in outs:
        np.testing.assert_array_equal(i, ei)
        np.testing.assert_array_equal(bits(v), bits(ev))


@pytest.mark.parametrize("light", [False, True])
@pytest.mark.parametrize("op", ["min", "max"])
@pytest.mark.parametrize("dtype", ["float32", "int32"])
def test_batch_key_modes(cuda, native, oracle_lib, dtype, op, light):
    """int32 values and range maximum on full and light plans: leftmost
    best index and its exact value, every path."""
    from rtxrmq_gb300.batch import RMQBatch
    starts, lengths, qstarts, qcounts, Af, Q = small_ragged(7, ties=True, align=1)
    A = (Af - 32).astype(np.int32) if dtype == "int32" else (Af - 32).astype(np.float32)
    A[::97] = -0.0 if dtype == "float32" else A[::97]  # signed zeros among ties
    key = A.astype(np.float32)
    _, ei = expected(oracle_lib, starts, lengths, qstarts, qcounts,
                     -key if op == "max" else key, Q)
    own = owned_mask(qstarts, qcounts, len(Q))
    offs = np.zeros(len(Q), np.int64)
    for s, qs, qc in zip(starts, qstarts, qcounts):
        offs[qs:qs + qc] = s
    cfg = [64, 256, 1024, 4096] * 8
    with RMQBatch(starts, lengths, qstarts, qcounts, cfg, op=op, dtype=dtype, light=light) as b:
        outs = run_all(cuda, b, A, Q)
    for v, i in outs:
        assert v.dtype == A.dtype
        np.testing.assert_array_equal(i[own], ei[own])
        np.testing.assert_array_equal(v[own].view(np.uint32),
                                      A[offs[own] + i[own]].view(np.uint32))


def test_batch_light_graph_capture(cuda, native, oracle_lib):
    """A light plan's run captured in a CUDA graph and replayed on new
    values gives the oracle's answers for those values."""
    import torch

    from rtxrmq_gb300.batch import RMQBatch
    starts, lengths, qstarts, qcounts, A, Q = small_ragged(5)
    own = owned_mask(qstarts, qcounts, len(Q))
    dA = torch.from_numpy(A).to(cuda)
    dQ = torch.from_numpy(Q).to(cuda)
    with RMQBatch(starts, lengths, qstarts, qcounts, light=True) as b:
        v = torch.empty(len(Q), dtype=torch.float32, device=cuda)
        i = torch.empty(len(Q), dtype=torch.int32, device=cuda)
        s = torch.cuda.Stream()
        with torch.cuda.stream(s):
            b.run(dA, dQ, v, i, stream=s)  # warm: kernel attributes set before capture
        s.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s):
            b.run(dA, dQ, v, i, stream=s)
        A2 = np.ascontiguousarray(A[::-1])
        dA.copy_(torch.from_numpy(A2))
        g.replay()
        torch.cuda.synchronize()
        ev, ei = expected(oracle_lib, starts, lengths, qstarts, qcounts, A2, Q)
        np.testing.assert_array_equal(i.cpu().numpy()[own], ei[own])
        np.testing.assert_array_equal(bits(v.cpu().numpy()[own]), bits(ev[own]))


def test_batch_modes_rejections(cuda, native):
    """Light block sizes that are not multiples of 32 or below 64, unknown
    flags, values of the wrong dtype, and a gradient of an int32 plan."""
    import torch

    import rtxrmq_gb300 as R
    from rtxrmq_gb300.batch import RMQBatch
    args = ([0, 100], [100, 50], [0, 10], [10, 5])
    for bad in (100, 32, 48):
        with pytest.raises(R.RMQError):
            RMQBatch(*args, [bad] * 32, light=True)
    with pytest.raises(ValueError):
        RMQBatch(*args, op="median")
    with RMQBatch(*args, dtype="int32") as b:
        vals = torch.zeros(150, dtype=torch.float32, device=cuda)
        q = torch.zeros((15, 2), dtype=torch.int32, device=cuda)
        with pytest.raises(TypeError):
            b.run(vals, q)
        v, i = b.run(vals.to(torch.int32), q)
        assert v.dtype == torch.int32
        with pytest.raises(R.RMQError):
            b.scatter_grad(i, torch.zeros(15, device=cuda), torch.zeros(150, device=cuda))


def test_batch_light_autotune(cuda, native, oracle_lib, tmp_path):
    """The whole-tile autotuner on a light plan picks light-valid block
    sizes, and the tuned plan answers like the oracle."""
    import torch

    from rtxrmq_gb300.batch import RMQBatch, autotune
    starts, lengths, qstarts, qcounts, A, Q = small_ragged(6)
    dA = torch.from_numpy(A).to(cuda)
    dQ = torch.from_numpy(Q).to(cuda)
    cfg = autotune(starts, lengths, qstarts, qcounts, dA, dQ, reps=1, cache=tmp_path / "c.json",
                   tiles=True, light=True)
    for bs, qc, lc in cfg:
        assert bs == 0 or (bs >= 64 and bs % 32 == 0)
    ev, ei = expected(oracle_lib, starts, lengths, qstarts, qcounts, A, Q)
    own = owned_mask(qstarts, qcounts, len(Q))
    with RMQBatch(starts, lengths, qstarts, qcounts, cfg, light=True) as b:
        v, i = b.run(dA, dQ)
        torch.cuda.synchronize()
    np.testing.assert_array_equal(i.cpu().numpy()[own], ei[own])
    np.testing.assert_array_equal(bits(v.cpu().numpy()[own]), bits(ev[own]))


@pytest.mark.parametrize("light", [False, True])
@pytest.mark.parametrize("op", ["min", "max"])
def test_batch_nan_and_signed_zero_order(cuda, native, op, light):
    """Batched plans over arrays holding quiet and signaling NaNs and +-0:
    the same order as the plain index (NaN last, canonical NaN returned,
    -0 == +0 leftmost), every path."""
    from test_gpu_light import expect_nan_case, nan_case

    from rtxrmq_gb300.batch import RMQBatch
    A, Qall = nan_case(21 + light, 12011)
    # three arrays over the buffer at odd offsets, each with its own queries
    starts = np.array([0, 4001, 8003], np.int64)
    lengths = np.array([4000, 4001, 4007], np.int64)
    qs, ev_all, ei_all = [], [], []
    for s, n in zip(starts, lengths):
        Q = Qall[(Qall[:, 1] < n)][:6000]
        ei, ev = expect_nan_case(A[s:s + n], Q, op)
        qs.append(Q)
        ei_all.append(ei)
        ev_all.append(ev)
    qcounts = np.array([len(q) for q in qs], np.int64)
    qstarts = np.concatenate([[0], np.cumsum(qcounts)[:-1]]).astype(np.int64)
    Q = np.concatenate(qs)
    ei, ev = np.concatenate(ei_all), np.concatenate(ev_all)
    with RMQBatch(starts, lengths, qstarts, qcounts, [64, 256, 1024, 4096] * 8, op=op,
                  light=light) as b:
        outs = run_all(cuda, b, A, Q)
    for v, i in outs:
        np.testing.assert_array_equal(i, ei)
        np.testing.assert_array_equal(v.view(np.uint32), ev)
