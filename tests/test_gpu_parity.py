"""GPU parity of the block-decomposition engine (alg 5 / 105) through the C
ABI, against the CPU oracle (restatement of the reference's BASE, pinned to
the reference's own outputs by tests/test_oracle_golden.py).

Bar: bit-exact values (the bits of A[idx]) and exact leftmost indices.
"""
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = sorted((Path(__file__).parent / "golden").glob("*.npz"))


def bits(x):
    return np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)


def run_index(cuda, A, Q, bs, values=True, indices=True, micro=True):
    """Build + query; micro=False forces the warp-scan path for queries
    inside one block (micro=True uses the sub-block level for every bs >= 64)."""
    import torch

    import rtxrmq_gb300 as R
    dA = torch.from_numpy(np.ascontiguousarray(A, dtype=np.float32)).to(cuda)
    dQ = torch.from_numpy(np.ascontiguousarray(Q, dtype=np.int32)).to(cuda)
    with R.RMQIndex(dA, bs, micro=micro) as ix:
        if micro and bs >= 64 and bs <= len(A):
            assert ix.info()["micro_levels"] > 0
        v, i = ix.query(dQ, values=values, indices=indices)
        torch.cuda.synchronize()
        return (None if v is None else v.cpu().numpy()), (None if i is None else i.cpu().numpy())


def assert_matches(A, Q, v, i, ev, ei):
    if i is not None:
        bad = np.nonzero(i != ei)[0]
        assert bad.size == 0, (f"{bad.size} index mismatches; first q={bad[0]} "
                               f"(l,r)={tuple(Q[bad[0]])} got {i[bad[0]]} want {ei[bad[0]]}")
    if v is not None:
        np.testing.assert_array_equal(bits(v), bits(ev))


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: p.stem)
@pytest.mark.parametrize("bs", [1, 2, 5, 32, 100, 1000, 4096, 1 << 15])
def test_golden_vectors(cuda, native, path, bs):
    """Engine output equals the reference's BASE outputs stored in the fixtures."""
    g = np.load(path)
    v, i = run_index(cuda, g["A"], g["Q"], bs)
    assert_matches(g["A"], g["Q"], v, i, g["base_val"], g["base_idx"])


def all_pairs(n):
    l, r = np.triu_indices(n)
    return np.stack([l, r], axis=1).astype(np.int32)


@pytest.mark.parametrize("micro", [True, False])
@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 31, 32, 33, 127, 300, 1000])
def test_exhaustive_small(cuda, native, oracle_lib, n, micro):
    """Every (l, r) of small tie-heavy arrays, across block sizes that put
    block edges everywhere (bs = 1 .. n), with and without the sub-block level."""
    import rtxrmq_gb300 as R
    A = R.gen_values_int(n, 4, n)
    Q = all_pairs(n)
    ev, ei = oracle_lib.base_val(A, Q), oracle_lib.base_idx(A, Q)
    for bs in sorted({1, 2, 3, 4, 7, 8, 16, 31, 32, 33, 64, 96, 100, 128, 160, 256, 512, n,
                      max(1, n // 2)}):
        if bs > n:
            continue
        v, i = run_index(cuda, A, Q, bs, micro=micro)
        assert_matches(A, Q, v, i, ev, ei)


@pytest.mark.parametrize("micro", [True, False])
@pytest.mark.parametrize("bs", [1 << 10, 1 << 12, 1 << 15, 0, 977])
def test_config_small_range(cuda, native, oracle_lib, bs, micro):
    """n=1e6 uniform values (seed 1321), q=2^20 small-range (lr=-3) queries."""
    import rtxrmq_gb300 as R
    n, q = 10**6, 1 << 20
    A = R.gen_values_uniform(n, 1321)
    Q = R.gen_queries(q, n, -3, 1321)
    v, i = run_index(cuda, A, Q, bs, micro=micro)
    assert_matches(A, Q, v, i, oracle_lib.base_val(A, Q), oracle_lib.base_idx(A, Q))


@pytest.mark.parametrize("micro", [True, False])
@pytest.mark.parametrize("lr", [-1, -2, -3, 1, 32, 1024, 65536])
@pytest.mark.parametrize("bs", [1 << 10, 1 << 13, 1 << 16, 12207, 4000, 1 << 18, 1 << 20])
def test_length_modes_medium(cuda, native, oracle_lib, lr, bs, micro):
    """n=2^22: every length mode and block-size class; oracle = the CPU
    restatement of RTX_blocks (exact, O(bs + nb) per query)."""
    import rtxrmq_gb300 as R
    n, q = 1 << 22, 1 << 16
    A = R.gen_values_uniform(n, 11)
    Q = R.gen_queries(q, n, lr, 100 + lr)
    v, i = run_index(cuda, A, Q, bs, micro=micro)
    ev, ei = oracle_lib.Blocks(A, 1 << 12).query(Q)
    assert_matches(A, Q, v, i, ev, ei)


@pytest.mark.parametrize("bs", [(1 << 22) + 5, 1 << 23])
@pytest.mark.parametrize("ties", [False, True])
def test_huge_blocks_wide_offsets(cuda, native, oracle_lib, bs, ties):
    """Blocks of 2^22+ elements: the micro table has 18+ levels, so its
    offsets are 4 bytes wide; queries inside one block span up to the whole
    block (every table level), on tie-free and tie-heavy values."""
    import torch

    import rtxrmq_gb300 as R
    n = (1 << 24) + 12345
    A = R.gen_values_int(n, 16, 5) if ties else R.gen_values_uniform(n, 5)
    Q = np.concatenate([R.gen_queries(1 << 12, n, length, 9 + k)
                        for k, length in enumerate((-2, 1 << 16, 1 << 20, (1 << 22) - 100))])
    with R.RMQIndex(torch.from_numpy(A).to(cuda), bs) as ix:
        assert ix.info()["micro_levels"] >= 18
    v, i = run_index(cuda, A, Q, bs)
    ev, ei = oracle_lib.Blocks(A, 1 << 12).query(Q)
    assert_matches(A, Q, v, i, ev, ei)


@pytest.mark.parametrize("micro", [True, False])
@pytest.mark.parametrize("length", [1, 32, 33, 1 << 10, 1 << 16, 1 << 20])
def test_tie_heavy(cuda, native, oracle_lib, length, micro):
    """Integers in [0,256): most ranges hold many equal minima; leftmost."""
    import rtxrmq_gb300 as R
    n, q = 1 << 23, 1 << 15
    A = R.gen_values_int(n, 256, 3)
    Q = R.gen_queries(q, n, length, 7)
    ev, ei = oracle_lib.Blocks(A, 1 << 12).query(Q)
    for bs in (1 << 10, 1 << 16):
        v, i = run_index(cuda, A, Q, bs, micro=micro)
        assert_matches(A, Q, v, i, ev, ei)


def test_special_values(cuda, native, oracle_lib):
    """+-0 compare equal (leftmost wins, its own sign returned), +-inf,
    subnormals, negatives."""
    rng = np.random.default_rng(0)
    n = 50_000
    A = rng.standard_normal(n).astype(np.float32)
    for val, cnt in ((0.0, 3000), (-0.0, 3000), (np.inf, 100), (-np.inf, 100), (1e-42, 100)):
        A[rng.integers(0, n, cnt)] = val
    import rtxrmq_gb300 as R
    Q = np.concatenate([R.gen_queries(20000, n, L, L) for L in (1, 2, 9, 333, 4000)])
    ev, ei = oracle_lib.base_val(A, Q), oracle_lib.base_idx(A, Q)
    for bs in (1, 64, 1024, 50_000):
        v, i = run_index(cuda, A, Q, bs)
        assert_matches(A, Q, v, i, ev, ei)
    # only zeros: every answer is the leftmost zero with its own sign
    Z = np.where(rng.random(4096) < 0.5, np.float32(0.0), np.float32(-0.0)).astype(np.float32)
    Qz = all_pairs(200)
    v, i = run_index(cuda, Z, Qz, 16)
    np.testing.assert_array_equal(i, Qz[:, 0])
    np.testing.assert_array_equal(bits(v), bits(Z[Qz[:, 0]]))


def test_outputs_optional(cuda, native, oracle_lib):
    import rtxrmq_gb300 as R
    n = 10_000
    A = R.gen_values_uniform(n, 4)
    Q = R.gen_queries(5000, n, -1, 4)
    v, i = run_index(cuda, A, Q, 100, values=True, indices=False)
    assert i is None
    np.testing.assert_array_equal(bits(v), bits(oracle_lib.base_val(A, Q)))
    v, i = run_index(cuda, A, Q, 100, values=False, indices=True)
    assert v is None
    np.testing.assert_array_equal(i, oracle_lib.base_idx(A, Q))


def test_unaligned_values(cuda, native, oracle_lib):
    """A values pointer that is not 16-byte aligned takes the scalar-load path."""
    import torch

    import rtxrmq_gb300 as R
    n = 70_001
    A = R.gen_values_int(n + 3, 50, 9)
    Q = R.gen_queries(20000, n, -3, 2)
    Q = np.concatenate([Q, R.gen_queries(5000, n, -1, 3)])
    big = torch.from_numpy(A).to(cuda)
    for off in (1, 2, 3):
        for bs in (1000, 1024):
            dA = big[off:off + n]
            dQ = torch.from_numpy(Q).to(cuda)
            with R.RMQIndex(dA, bs) as ix:
                assert ix.info()["aligned"] == 0
                v, i = ix.query(dQ)
                torch.cuda.synchronize()
            Ah = A[off:off + n]
            np.testing.assert_array_equal(i.cpu().numpy(), oracle_lib.base_idx(Ah, Q))
            np.testing.assert_array_equal(bits(v.cpu().numpy()), bits(oracle_lib.base_val(Ah, Q)))


def test_invalid_queries(cuda, native):
    """l > r, r >= n, l < 0: idx -1, NaN value, counted; valid ones unaffected."""
    import torch

    import rtxrmq_gb300 as R
    n = 1000
    A = R.gen_values_uniform(n, 1)
    Q = np.array([[0, 999], [5, 4], [0, 1000], [-1, 3], [10, 10], [999, 999], [2**31 - 1, 2**31 - 1]],
                 dtype=np.int32)
    dA = torch.from_numpy(A).to(cuda)
    with R.RMQIndex(dA, 64) as ix:
        v, i = ix.query(torch.from_numpy(Q).to(cuda))
        assert ix.invalid_count() == 4
        v, i = v.cpu().numpy(), i.cpu().numpy()
    assert list(i) == [int(np.argmin(A)), -1, -1, -1, 10, 999, -1]
    assert np.isnan(v[[1, 2, 3, 6]]).all()
    assert v[0] == A.min()


def test_gpu_base_matches_oracle(cuda, native, oracle_lib):
    """alg 2 / 102 (GPU brute force) equals BASE, including on the fixtures."""
    import torch

    import rtxrmq_gb300 as R
    for path in GOLDEN:
        g = np.load(path)
        dA = torch.from_numpy(g["A"]).to(cuda)
        dQ = torch.from_numpy(g["Q"]).to(cuda)
        q = len(g["Q"])
        np.testing.assert_array_equal(R.gpu_rmq_basic_idx(len(g["A"]), q, dA, dQ), g["base_idx"])
        np.testing.assert_array_equal(bits(R.gpu_rmq_basic(len(g["A"]), q, dA, dQ)), bits(g["base_val"]))


def test_rtx_rmq_mirror(cuda, native, oracle_lib):
    """rtx_rmq(alg, n, bs, q, dA, dQ) mirrors src/rtx.h:24-177 for 5 / 105."""
    import torch

    import rtxrmq_gb300 as R
    n, q = 50_000, 20_000
    A = R.gen_values_uniform(n, 8)
    Q = R.gen_queries(q, n, -2, 8)
    dA, dQ = torch.from_numpy(A).to(cuda), torch.from_numpy(Q).to(cuda)
    vals = R.rtx_rmq(5, n, R.bs_from_nb(n, 512), q, dA, dQ, reps=2)
    idx = R.rtx_rmq(105, n, 1 << 10, q, dA, dQ)
    assert vals.dtype == np.float32 and idx.dtype == np.int32
    np.testing.assert_array_equal(bits(vals), bits(oracle_lib.base_val(A, Q)))
    np.testing.assert_array_equal(idx, oracle_lib.base_idx(A, Q))
    with pytest.raises(R.RMQError):
        R.rtx_rmq(3, n, 1024, q, dA, dQ)


def test_cli_check_passes(native):
    """The CLI's --check (src/main.cu:140-167) passes for algs 5 and 105."""
    import subprocess
    cli = Path(__file__).resolve().parent.parent / "rtxrmq_gb300" / "_lib" / "rtxrmq"
    for alg in ("5", "105", "2", "102"):
        r = subprocess.run([str(cli), "200000", "100000", "-3", alg, "--bs", "1024", "--reps", "2",
                            "--seed", "1321", "--check", "--nt", "4"],
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0 and "pass" in r.stdout, r.stdout + r.stderr


def test_query_host_buffers(cuda, native, oracle_lib):
    """rmq_query_host: pinned and pageable host buffers, streamed through the
    staged pipeline (several chunks: q > one 4 Mi-query chunk is exercised by
    the full-size bench); device buffers are passed through."""
    import torch

    import rtxrmq_gb300 as R
    n, q = 200_000, 100_000
    A = R.gen_values_uniform(n, 12)
    Q = R.gen_queries(q, n, -2, 12)
    ev, ei = oracle_lib.base_val(A, Q), oracle_lib.base_idx(A, Q)
    with R.RMQIndex(torch.from_numpy(A).to(cuda), 1024) as ix:
        hQ = torch.from_numpy(Q).pin_memory()
        hV = torch.empty(q, dtype=torch.float32).pin_memory()
        hI = torch.empty(q, dtype=torch.int32).pin_memory()
        ix.query_host(hQ, hV, hI)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(hI.numpy(), ei)
        np.testing.assert_array_equal(bits(hV.numpy()), bits(ev))
        ix.query_host(hQ, None, hI)  # index mode only
        torch.cuda.synchronize()
        np.testing.assert_array_equal(hI.numpy(), ei)
        v = np.full(q, np.nan, np.float32)
        i = np.full(q, -7, np.int32)
        ix.query_host(Q, v, i)  # pageable numpy buffers
        torch.cuda.synchronize()
        np.testing.assert_array_equal(i, ei)
        np.testing.assert_array_equal(bits(v), bits(ev))
        dv = torch.empty(q, dtype=torch.float32, device=cuda)
        di = torch.empty(q, dtype=torch.int32, device=cuda)
        ix.query_host(torch.from_numpy(Q).to(cuda), dv, di)  # device buffers pass through
        torch.cuda.synchronize()
        np.testing.assert_array_equal(di.cpu().numpy(), ei)


def test_query_host_many_chunks(cuda, native, oracle_lib):
    """More queries than three staging chunks (4 Mi queries each), values
    only and indices only, against the device path."""
    import torch

    import rtxrmq_gb300 as R
    n, q = 1 << 22, (3 << 22) + 12345
    A = R.gen_values_int(n, 5000, 21)
    Q = R.gen_queries(q, n, -3, 21)
    with R.RMQIndex(torch.from_numpy(A).to(cuda), 4096) as ix:
        dv, di = ix.query(torch.from_numpy(Q).to(cuda))
        hQ = torch.from_numpy(Q).pin_memory()
        hv = torch.empty(q, dtype=torch.float32).pin_memory()
        hi = torch.empty(q, dtype=torch.int32).pin_memory()
        ix.query_host(hQ, hv, hi)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(hi.numpy(), di.cpu().numpy())
        np.testing.assert_array_equal(bits(hv.numpy()), bits(dv.cpu().numpy()))
        hi2 = torch.full((q,), -9, dtype=torch.int32).pin_memory()
        ix.query_host(hQ, None, hi2)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(hi2.numpy(), di.cpu().numpy())


def test_query_host_staged_path(cuda, native, oracle_lib, monkeypatch):
    """The staged host path (device staging, query copies or in-place reads,
    result copies overlapping later chunks) gives the same results; forced
    with RTXRMQ_HOST_STAGED=1 because buffers here are addressable."""
    import torch

    import rtxrmq_gb300 as R
    monkeypatch.setenv("RTXRMQ_HOST_STAGED", "1")
    n, q = 1 << 21, (1 << 23) + 777  # three chunks
    A = R.gen_values_int(n, 3000, 31)
    Q = R.gen_queries(q, n, -3, 31)
    with R.RMQIndex(torch.from_numpy(A).to(cuda), 2048) as ix:
        dv, di = ix.query(torch.from_numpy(Q).to(cuda))
        dv, di = dv.cpu().numpy(), di.cpu().numpy()
        for pinned in (True, False):
            hQ = torch.from_numpy(Q)
            hv = torch.empty(q, dtype=torch.float32)
            hi = torch.empty(q, dtype=torch.int32)
            if pinned:
                hQ, hv, hi = hQ.pin_memory(), hv.pin_memory(), hi.pin_memory()
            ix.query_host(hQ, hv, hi)
            torch.cuda.synchronize()
            np.testing.assert_array_equal(hi.numpy(), di)
            np.testing.assert_array_equal(bits(hv.numpy()), bits(dv))


def test_query_host_staged_two_streams(cuda, native, oracle_lib, monkeypatch):
    """Two staged host calls on one handle from two streams, enqueued back to
    back: the second call's chunks reuse staging slots only after the first
    call's kernels and copies are done with them."""
    import torch

    import rtxrmq_gb300 as R
    monkeypatch.setenv("RTXRMQ_HOST_STAGED", "1")
    n = 1 << 21
    A = R.gen_values_uniform(n, 41)
    Q1 = R.gen_queries((1 << 24) + 5, n, -1, 41)   # five chunks
    Q2 = R.gen_queries((1 << 22) + 3, n, -3, 42)   # two chunks
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    with R.RMQIndex(torch.from_numpy(A).to(cuda), 4096) as ix:
        want = []
        for Q in (Q1, Q2):
            dv, di = ix.query(torch.from_numpy(Q).to(cuda))
            want.append((dv.cpu().numpy(), di.cpu().numpy()))
        torch.cuda.synchronize()
        outs = []
        for Q, s in ((Q1, s1), (Q2, s2)):
            hv = torch.empty(len(Q), dtype=torch.float32)
            hi = torch.empty(len(Q), dtype=torch.int32)
            ix.query_host(torch.from_numpy(Q), hv, hi, stream=s)
            outs.append((hv, hi))
        s1.synchronize()
        s2.synchronize()
        for (hv, hi), (dv, di) in zip(outs, want):
            np.testing.assert_array_equal(hi.numpy(), di)
            np.testing.assert_array_equal(bits(hv.numpy()), bits(dv))


def test_save_load_index(cuda, native, oracle_lib, tmp_path):
    """rmq_save / rmq_load (the role of HRMQ's saveDS / loadDS): a loaded
    index answers like the built one; other values, lengths, foreign or
    truncated files are refused."""
    import torch

    import rtxrmq_gb300 as R
    n = 300_001
    A = R.gen_values_int(n, 999, 41)
    Q = np.concatenate([R.gen_queries(50_000, n, L, 41) for L in (-1, -3, 1, 40)])
    dA = torch.from_numpy(A).to(cuda)
    dQ = torch.from_numpy(Q).to(cuda)
    ev, ei = oracle_lib.base_val(A, Q), oracle_lib.base_idx(A, Q)
    for bs, micro in ((1024, True), (1024, False), (1000, True), (1, True)):
        path = tmp_path / f"ix_{bs}_{micro}.rmq"
        with R.RMQIndex(dA, bs, micro=micro) as ix:
            ix.save(path)
            info = ix.info()
        with R.RMQIndex.load(dA, path) as ix2:
            assert ix2.info()["struct_bytes"] == info["struct_bytes"]
            assert ix2.info()["micro_levels"] == info["micro_levels"]
            v, i = ix2.query(dQ)
            torch.cuda.synchronize()
            np.testing.assert_array_equal(i.cpu().numpy(), ei)
            np.testing.assert_array_equal(bits(v.cpu().numpy()), bits(ev))
    path = tmp_path / "ix_1024_True.rmq"
    B = A.copy()
    B[12345] += 1.0
    with pytest.raises(R.RMQError, match="values differ"):
        R.RMQIndex.load(torch.from_numpy(B).to(cuda), path)
    with pytest.raises(R.RMQError, match="n="):
        R.RMQIndex.load(dA[:-1].contiguous(), path)
    raw = path.read_bytes()
    (tmp_path / "trunc.rmq").write_bytes(raw[:len(raw) // 2])
    with pytest.raises(R.RMQError, match="truncated"):
        R.RMQIndex.load(dA, tmp_path / "trunc.rmq")
    bad = bytearray(raw)
    bad[20] ^= 0xFF
    (tmp_path / "bad.rmq").write_bytes(bytes(bad))
    with pytest.raises(R.RMQError, match="not an index file"):
        R.RMQIndex.load(dA, tmp_path / "bad.rmq")


def np_leftmost(A, Q, op):
    """Brute-force leftmost argmin / argmax (numpy's first occurrence)."""
    f = np.argmin if op == "min" else np.argmax
    return np.array([l + f(A[l:r + 1]) for l, r in Q], dtype=np.int32)


@pytest.mark.parametrize("dtype", ["float32", "int32"])
@pytest.mark.parametrize("op", ["min", "max"])
@pytest.mark.parametrize("micro", [True, False])
def test_key_modes(cuda, native, dtype, op, micro):
    """Range maximum and int32 elements (the role of HRMQ's integer
    constructors): leftmost best, exact values, every block-size class."""
    import torch

    import rtxrmq_gb300 as R
    rng = np.random.default_rng(77)
    n = 5000
    if dtype == "int32":
        A = rng.integers(-2**31, 2**31 - 1, n, dtype=np.int64).astype(np.int32)
        A[rng.integers(0, n, 500)] = rng.integers(-3, 3, 500)  # ties, around zero
        A[rng.integers(0, n, 20)] = np.iinfo(np.int32).max
        A[rng.integers(0, n, 20)] = np.iinfo(np.int32).min
    else:
        A = rng.standard_normal(n).astype(np.float32)
        A[rng.integers(0, n, 300)] = 0.0
        A[rng.integers(0, n, 300)] = -0.0
        A[rng.integers(0, n, 20)] = np.inf
        A[rng.integers(0, n, 20)] = -np.inf
    Q = np.concatenate([R.gen_queries(1500, n, L, 5 + L) for L in (-1, -3, 1, 2, 31, 33, 100, 700)])
    ei = np_leftmost(A, Q, op)
    dA = torch.from_numpy(A).to(cuda)
    dQ = torch.from_numpy(Q).to(cuda)
    for bs in (1, 7, 64, 96, 1024, n):
        with R.RMQIndex(dA, bs, micro=micro, op=op) as ix:
            inf = ix.info()
            assert inf["is_max"] == (op == "max") and inf["is_int32"] == (dtype == "int32")
            v, i = ix.query(dQ)
            torch.cuda.synchronize()
            i, v = i.cpu().numpy(), v.cpu().numpy()
        np.testing.assert_array_equal(i, ei)
        np.testing.assert_array_equal(v.view(np.uint32), A[ei].view(np.uint32))


def random_case(seed):
    """One seeded random configuration: size, block size, element type, min /
    max, sub-block level on / off, values pointer offset (unaligned for
    offsets 1-3), value distribution and a mix of query lengths."""
    import rtxrmq_gb300 as R
    rng = np.random.default_rng(1000 + seed)
    edge_sizes = [1, 2, 31, 32, 33, 63, 64, 65, 95, 96, 97, 1000, 4095, 4096, 4097]
    n = int(rng.choice(edge_sizes)) if rng.random() < 0.4 else int(rng.integers(1, 200_000))
    if rng.random() < 0.5:
        bs = int(rng.integers(1, n + 1))
    else:
        bs = min(n, int(rng.choice([1, 16, 32, 33, 64, 96, 1024, 4096, 65536])))
    dtype = str(rng.choice(["float32", "int32"]))
    op = str(rng.choice(["min", "max"]))
    micro = bool(rng.random() < 0.7)
    off = int(rng.integers(0, 4))
    kind = int(rng.integers(0, 3))
    if dtype == "float32":
        A = (rng.random(n).astype(np.float32) if kind == 0 else
             rng.integers(0, 8, n).astype(np.float32) if kind == 1 else
             rng.standard_normal(n).astype(np.float32))
        if kind == 2:
            A[rng.integers(0, n, max(1, n // 50))] = -0.0
    else:
        A = (rng.integers(-2**31, 2**31 - 1, n, dtype=np.int64).astype(np.int32) if kind == 0 else
             rng.integers(-4, 4, n).astype(np.int32))
    qs = [R.gen_queries(600, n, L, seed + k) for k, L in enumerate((-1, -2, -3))]
    qs += [R.gen_queries(300, n, L, seed + 10 + k) for k, L in
           enumerate((1, 2, 31, 32, 33, 64, 1000)) if L <= n]
    qs.append(np.array([[0, n - 1], [n - 1, n - 1], [0, 0]], dtype=np.int32))
    return n, bs, dtype, op, micro, off, A, np.concatenate(qs)


@pytest.mark.parametrize("seed", range(64))
def test_random_configurations(cuda, native, seed):
    """Seeded random configurations (random_case) against a brute-force
    leftmost argmin / argmax, values compared as bits."""
    import torch

    import rtxrmq_gb300 as R
    n, bs, dtype, op, micro, off, A, Q = random_case(seed)
    ei = np_leftmost(A, Q, op)
    pad = np.zeros(off, dtype=A.dtype)
    big = torch.from_numpy(np.concatenate([pad, A])).to(cuda)
    dA = big[off:off + n]
    with R.RMQIndex(dA, bs, micro=micro, op=op) as ix:
        assert ix.info()["aligned"] == (1 if off == 0 else 0)
        v, i = ix.query(torch.from_numpy(Q).to(cuda))
        torch.cuda.synchronize()
        i, v = i.cpu().numpy(), v.cpu().numpy()
    cfg = f"n={n} bs={bs} {dtype} {op} micro={micro} off={off}"
    bad = np.nonzero(i != ei)[0]
    assert bad.size == 0, f"{cfg}: {bad.size} index mismatches, first {tuple(Q[bad[0]])}"
    np.testing.assert_array_equal(v.view(np.uint32), A[ei].view(np.uint32), err_msg=cfg)


def test_probe_gather(cuda, native, oracle_lib):
    """rmq_probe_gather (the random-access ceiling the bench times beside
    rmq_query) reads suf[l] and pre[r] only: exact for queries whose ends lie
    in adjacent blocks, clamped (no fault, no error) for out-of-range ones."""
    import torch

    import oracle
    import rtxrmq_gb300 as R
    rng = np.random.default_rng(11)
    n, bs = 100_000, 1000
    A = rng.integers(0, 64, n).astype(np.float32)  # many ties
    lb = rng.integers(0, n // bs - 1, 20_000)
    l = lb * bs + rng.integers(0, bs, lb.size)
    r = (lb + 1) * bs + rng.integers(0, bs, lb.size)
    Q = np.stack([l, r], axis=1).astype(np.int32)
    ev, ei = oracle.base_val(A, Q), oracle.base_idx(A, Q)
    dA = torch.from_numpy(A).to(cuda)
    with R.RMQIndex(dA, bs) as ix:
        v, i = ix.probe_gather(torch.from_numpy(Q).to(cuda))
        bad = torch.tensor([[-5, 3], [7, n + 100], [n + 1, n + 2]], dtype=torch.int32, device=cuda)
        vb, ib = ix.probe_gather(bad)
        torch.cuda.synchronize()
        assert ix.invalid_count() == 0
    assert_matches(A, Q, v.cpu().numpy(), i.cpu().numpy(), ev, ei)
    ib = ib.cpu().numpy()
    assert ((ib >= 0) & (ib < n)).all()


def test_allocation_failure_injection(cuda, native, oracle_lib, monkeypatch, tmp_path):
    """Host-side fault injection (RTXRMQ_FAIL_ALLOC=1 makes every device
    allocation of the library fail as out-of-memory): each allocating call
    returns RMQ_ENOMEM with a message, nothing leaks or breaks, and the same
    calls succeed once the variable is cleared. No GPU fault is involved."""
    import torch

    import oracle
    import rtxrmq_gb300 as R
    from rtxrmq_gb300._native import RMQ_ENOMEM
    from rtxrmq_gb300.batch import RMQBatch
    rng = np.random.default_rng(3)
    A = rng.random(20000).astype(np.float32)
    Q = R.gen_queries(5000, len(A), -3, 4)
    dA = torch.from_numpy(A).to(cuda)
    ei = oracle.base_idx(A, Q)
    with R.RMQIndex(dA, 1024) as ix:
        ix.save(tmp_path / "ix.rmq")
        monkeypatch.setenv("RTXRMQ_FAIL_ALLOC", "1")
        with pytest.raises(R.RMQError) as e:
            R.RMQIndex(dA, 1024)
        assert e.value.code == RMQ_ENOMEM and "failed" in str(e.value)
        with pytest.raises(R.RMQError):
            RMQBatch([0], [len(A)], [0], [len(Q)])
        with pytest.raises(R.RMQError):
            R.RMQIndex.load(dA, tmp_path / "ix.rmq")
        monkeypatch.setenv("RTXRMQ_HOST_STAGED", "1")  # needs its staging allocation
        hv, hi = np.empty(len(Q), np.float32), np.empty(len(Q), np.int32)
        with pytest.raises(R.RMQError):
            ix.query_host(Q, hv, hi)
        # the existing index is untouched and answers on the device
        v, i = ix.query(torch.from_numpy(Q).to(cuda))
        np.testing.assert_array_equal(i.cpu().numpy(), ei)
        monkeypatch.delenv("RTXRMQ_FAIL_ALLOC")
        ix.query_host(Q, hv, hi)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(hi, ei)
    with R.RMQIndex.load(dA, tmp_path / "ix.rmq") as ix2:
        v, i = ix2.query(torch.from_numpy(Q).to(cuda))
        np.testing.assert_array_equal(i.cpu().numpy(), ei)


def test_query_graph_capture(cuda, native, oracle_lib):
    """rmq_query allocates nothing, so it can be captured in a CUDA graph
    (after a first call has cached its launch configuration) and replayed on
    new query contents."""
    import torch

    import oracle
    import rtxrmq_gb300 as R
    rng = np.random.default_rng(21)
    n = 200_000
    A = rng.random(n).astype(np.float32)
    dA = torch.from_numpy(A).to(cuda)
    Q0 = R.gen_queries(50_000, n, -3, 1)
    dQ = torch.from_numpy(Q0).to(cuda)
    with R.RMQIndex(dA, 1024) as ix:
        v = torch.empty(len(Q0), dtype=torch.float32, device=cuda)
        i = torch.empty(len(Q0), dtype=torch.int32, device=cuda)
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            ix.query(dQ, out_val=v, out_idx=i, stream=s)  # warm: caches the launch shape
        torch.cuda.current_stream().wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            ix.query(dQ, out_val=v, out_idx=i)
        for seed, lr in ((2, -1), (3, 1024), (4, -3)):
            Q = R.gen_queries(len(Q0), n, lr, seed)
            dQ.copy_(torch.from_numpy(Q).to(cuda))
            g.replay()
            torch.cuda.synchronize()
            np.testing.assert_array_equal(i.cpu().numpy(), oracle.base_idx(A, Q))
            np.testing.assert_array_equal(v.cpu().numpy().view(np.uint32),
                                          oracle.base_val(A, Q).view(np.uint32))


def test_concurrent_queries_one_handle(cuda, native, oracle_lib):
    """A handle is immutable after its build: host threads may query it at
    the same time on their own streams (device and host-buffer paths)."""
    import threading

    import torch

    import oracle
    import rtxrmq_gb300 as R
    rng = np.random.default_rng(22)
    n = 300_000
    A = rng.integers(0, 1000, n).astype(np.float32)
    dA = torch.from_numpy(A).to(cuda)
    sets = [R.gen_queries(40_000, n, lr, 30 + k) for k, lr in enumerate((-1, -3, 64, -2))]
    want = [oracle.base_idx(A, Q) for Q in sets]
    got = [None] * len(sets)
    errors = []
    with R.RMQIndex(dA, 2048) as ix:
        def work(k):
            try:
                torch.cuda.set_device(cuda)
                s = torch.cuda.Stream()
                with torch.cuda.stream(s):
                    if k % 2 == 0:
                        v, i = ix.query(torch.from_numpy(sets[k]).to(cuda), stream=s)
                        s.synchronize()
                        got[k] = i.cpu().numpy()
                    else:
                        hv = np.empty(len(sets[k]), np.float32)
                        hi = np.empty(len(sets[k]), np.int32)
                        for _ in range(3):
                            ix.query_host(sets[k], hv, hi, stream=s)
                        s.synchronize()
                        got[k] = hi
            except Exception as e:  # surfaced below
                errors.append(e)
        threads = [threading.Thread(target=work, args=(k,)) for k in range(len(sets))]
        for t in threads:
            t.start()
        for t in threads:
            t.join(timeout=120)
        assert not errors, errors
        for k in range(len(sets)):
            np.testing.assert_array_equal(got[k], want[k])
        assert ix.invalid_count() == 0


def test_cli_csv_nb_and_power(native, tmp_path):
    """The CLI's --save-time row has the reference's 13 columns
    (dev,alg,reps,n,bs,q,lr,t,q/s,ns/q,construction,outbuffer,tempbuffer,
    scripts/perf-benchmark.sh:30) with bs resolved from --nb as n / nb
    (src/tools.h:129-132); --save-power writes a power table and prints
    RMQs/J (or warns and continues where NVML is unavailable)."""
    import subprocess
    cli = Path(__file__).resolve().parent.parent / "rtxrmq_gb300" / "_lib" / "rtxrmq"
    csv = tmp_path / "t.csv"
    pw = tmp_path / "p.dat"
    n, q, nb = 1_000_003, 262_144, 512
    for alg in ("5", "105"):
        r = subprocess.run([str(cli), str(n), str(q), "-1", alg, "--nb", str(nb), "--reps", "3",
                            f"--save-time={csv}", f"--save-power={pw}"],
                           capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "RMQs/J" in r.stdout or "power sampling unavailable" in r.stderr
    rows = [line.split(",") for line in csv.read_text().splitlines()]
    assert len(rows) == 2
    for row in rows:
        assert len(row) == 13
        dev, alg, reps, n_, bs, q_, lr = row[:7]
        assert (int(reps), int(n_), int(bs), int(q_), int(lr)) == (3, n, n // nb, q, -1)
        t, qps, nsq, constr = (float(x) for x in row[7:11])
        assert t > 0 and qps > 0 and nsq > 0 and constr > 0
        assert abs(qps * nsq / 1e9 - 1.0) < 1e-3   # q/s and ns/q are reciprocal
    if pw.exists():
        assert pw.stat().st_size > 0


def test_abi_argument_errors(cuda, native):
    """Every entry point rejects bad arguments with RMQ_EINVAL and a message,
    without launching anything: NULL pointers, sizes out of range, misaligned
    query / output buffers, NULL handles, malformed batch layouts."""
    import ctypes as C

    import torch

    from rtxrmq_gb300._native import RMQ_EINVAL
    L = native
    A = torch.rand(1000, device=cuda)
    Q = torch.zeros((10, 2), dtype=torch.int32, device=cuda)
    out = torch.empty(16, dtype=torch.int32, device=cuda)
    h = C.c_void_p()

    def einval(rc):
        assert rc == RMQ_EINVAL, rc
        assert L.rmq_last_error_string()

    einval(L.rmq_build(None, 1000, 64, None, C.byref(h)))
    einval(L.rmq_build(A.data_ptr(), 0, 64, None, C.byref(h)))
    einval(L.rmq_build(A.data_ptr(), 2**31, 64, None, C.byref(h)))
    einval(L.rmq_build(A.data_ptr(), 1000, 64, None, None))
    assert L.rmq_build(A.data_ptr(), 1000, 64, None, C.byref(h)) == 0
    try:
        einval(L.rmq_query(None, Q.data_ptr(), 10, None, out.data_ptr(), None))
        einval(L.rmq_query(h, Q.data_ptr(), -1, None, out.data_ptr(), None))
        einval(L.rmq_query(h, None, 10, None, out.data_ptr(), None))
        einval(L.rmq_query(h, Q.data_ptr() + 4, 10, None, out.data_ptr(), None))   # 8-byte queries
        einval(L.rmq_query(h, Q.data_ptr(), 10, None, None, None))                  # no output
        einval(L.rmq_query(h, Q.data_ptr(), 10, None, out.data_ptr() + 2, None))   # misaligned output
        einval(L.rmq_query_host(h, None, 10, None, out.data_ptr(), None))
        einval(L.rmq_probe_gather(h, Q.data_ptr() + 4, 10, None, out.data_ptr(), None))
        einval(L.rmq_info(h, None))
    finally:
        assert L.rmq_free(h) == 0
    einval(L.rmq_query_scan(A.data_ptr(), 0, Q.data_ptr(), 10, None, out.data_ptr(), None))
    b = C.c_void_p()
    i64 = lambda *v: (C.c_int64 * len(v))(*v)  # noqa: E731
    einval(L.rmq_batch_create(0, i64(0), i64(1), i64(0), i64(1), None, C.byref(b)))
    einval(L.rmq_batch_create(1, i64(0), i64(-5), i64(0), i64(1), None, C.byref(b)))
    einval(L.rmq_batch_create(1, i64(-1), i64(5), i64(0), i64(1), None, C.byref(b)))
    einval(L.rmq_batch_create(1, None, i64(5), i64(0), i64(1), None, C.byref(b)))
    einval(L.rmq_batch_run(None, A.data_ptr(), Q.data_ptr(), None, out.data_ptr(), None))
    einval(L.rmq_batch_scatter_grad(None, out.data_ptr(), A.data_ptr(), A.data_ptr(), 0, None))
