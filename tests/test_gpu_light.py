"""GPU parity of the light index (RMQ_BUILD_LIGHT: block and micro-block
tables only, no per-element prefix / suffix entries; a query the table
probe leaves open scans one line of values per end instead of reading an
entry), through the C ABI, against the oracle: bit-exact values and
leftmost indices, as for the full index."""
import numpy as np
import pytest

from test_gpu_parity import all_pairs, assert_matches, np_leftmost, random_case

pytestmark = pytest.mark.gpu


def run_light(cuda, A, Q, bs, op="min", off=0):
    import torch

    import rtxrmq_gb300 as R
    pad = np.zeros(off, dtype=A.dtype)
    big = torch.from_numpy(np.concatenate([pad, A])).to(cuda)
    dA = big[off:off + len(A)]
    with R.RMQIndex(dA, bs, light=True, op=op) as ix:
        info = ix.info()
        assert info["light"] == 1 and info["micro_levels"] > 0
        v, i = ix.query(torch.from_numpy(np.ascontiguousarray(Q, dtype=np.int32)).to(cuda))
        torch.cuda.synchronize()
        return v.cpu().numpy(), i.cpu().numpy(), info


@pytest.mark.parametrize("n", [64, 65, 95, 127, 300, 1000, 2049])
def test_light_exhaustive_small(cuda, native, oracle_lib, n):
    """Every (l, r) of small tie-heavy arrays for block sizes 64 .. n (and
    one block of n rounded up to a multiple of 32)."""
    import rtxrmq_gb300 as R
    A = R.gen_values_int(n, 4, n + 7)
    Q = all_pairs(n)
    ev, ei = oracle_lib.base_val(A, Q), oracle_lib.base_idx(A, Q)
    for bs in sorted({64, 96, 128, 160, 256, 512, 1024, (n + 31) // 32 * 32}):
        if bs > (n + 31) // 32 * 32:
            continue
        v, i, _ = run_light(cuda, A, Q, bs)
        assert_matches(A, Q, v, i, ev, ei)


@pytest.mark.parametrize("ties", [False, True])
@pytest.mark.parametrize("lr", [-1, -2, -3, 1, 32, 1024, 65536])
@pytest.mark.parametrize("bs", [64, 1 << 10, 1 << 13, 1 << 16])
def test_light_length_modes(cuda, native, oracle_lib, lr, bs, ties):
    """n=2^22 (+ a partial last block), every length mode, tie-free and
    tie-heavy values, against the oracle's decomposition."""
    import rtxrmq_gb300 as R
    n, q = (1 << 22) + 1000, 1 << 15
    A = R.gen_values_int(n, 64, 3) if ties else R.gen_values_uniform(n, 3)
    Q = R.gen_queries(q, n, lr, 200 + lr)
    v, i, info = run_light(cuda, A, Q, bs)
    # no per-element entries: tables only (the full index holds 32 bytes per
    # element; the block table over 64-element blocks alone is 2.4)
    assert info["struct_bytes"] < 4 * n
    ev, ei = oracle_lib.Blocks(A, 1 << 12).query(Q)
    assert_matches(A, Q, v, i, ev, ei)


@pytest.mark.parametrize("seed", range(24))
def test_light_random_configurations(cuda, native, seed):
    """The parity suite's seeded random configurations (element types,
    min / max, unaligned values, value distributions, query mixes) on the
    light index, with the block size rounded to a multiple of 32."""
    n, bs, dtype, op, micro, off, A, Q = random_case(seed)
    if n < 64:
        pytest.skip("a light index needs blocks of at least 64 elements")
    bs = max(64, bs // 32 * 32)
    ei = np_leftmost(A, Q, op)
    v, i, _ = run_light(cuda, A, Q, bs, op=op, off=off)
    bad = np.nonzero(i != ei)[0]
    assert bad.size == 0, f"n={n} bs={bs} {dtype} {op} off={off}: first {tuple(Q[bad[0]])}"
    np.testing.assert_array_equal(v.view(np.uint32), A[ei].view(np.uint32))


@pytest.mark.parametrize("off", [0, 1])
def test_light_special_values(cuda, native, oracle_lib, off):
    """Values whose micro-block minimum the build finds by key before index:
    +-0 mixed inside micro-blocks (leftmost wins with its own sign), +-inf,
    subnormals; int32 maximum over arrays mostly at INT_MIN (the largest
    key, the one past-the-end elements take) with a ragged last
    micro-block; aligned and unaligned values."""
    import rtxrmq_gb300 as R
    rng = np.random.default_rng(7 + off)
    n = 20_000 + 17
    A = rng.standard_normal(n).astype(np.float32)
    for val, cnt in ((0.0, 4000), (-0.0, 4000), (np.inf, 100), (-np.inf, 50), (1e-42, 100)):
        A[rng.integers(0, n, cnt)] = val
    Q = np.concatenate([R.gen_queries(20_000, n, L, L) for L in (1, 2, 9, 33, 333, 4000)] +
                       [np.array([[0, n - 1], [n - 40, n - 1], [n - 1, n - 1]], dtype=np.int32)])
    ev, ei = oracle_lib.base_val(A, Q), oracle_lib.base_idx(A, Q)
    for bs in (64, 1024, 20_032):
        v, i, _ = run_light(cuda, A, Q, bs, off=off)
        assert_matches(A, Q, v, i, ev, ei)
    # zeros only: every answer is the leftmost element, with its own sign
    Z = np.where(rng.random(1000 + 5) < 0.5, np.float32(0.0), np.float32(-0.0)).astype(np.float32)
    Qz = all_pairs(len(Z))
    v, i, _ = run_light(cuda, Z, Qz, 64, off=off)
    np.testing.assert_array_equal(i, Qz[:, 0])
    np.testing.assert_array_equal(v.view(np.uint32), Z[Qz[:, 0]].view(np.uint32))
    # int32 maximum, values mostly INT_MIN: ties at the largest key
    I = np.full(1000 + 13, np.iinfo(np.int32).min, dtype=np.int32)
    I[rng.integers(0, len(I), 20)] = rng.integers(-5, 5, 20)
    Qi = all_pairs(len(I))
    v, i, _ = run_light(cuda, I, Qi, 96, op="max", off=off)
    np.testing.assert_array_equal(i, np_leftmost(I, Qi, "max"))
    np.testing.assert_array_equal(v, I[i])


def test_light_invalid_save_load_and_rejections(cuda, native, oracle_lib, tmp_path):
    """Invalid queries, save / load of a light index, and the block sizes a
    light index refuses (not a multiple of 32, below 64, no sub-block level)."""
    import torch

    import rtxrmq_gb300 as R
    n = 100_000
    A = R.gen_values_uniform(n, 5)
    Q = R.gen_queries(20_000, n, -3, 6)
    Q[:3] = [[5, 4], [0, n], [-1, 2]]
    dA = torch.from_numpy(A).to(cuda)
    dQ = torch.from_numpy(Q).to(cuda)
    ei = oracle_lib.base_idx(A, Q)
    ei[:3] = -1
    with R.RMQIndex(dA, 2048, light=True) as ix:
        v, i = ix.query(dQ)
        np.testing.assert_array_equal(i.cpu().numpy(), ei)
        assert ix.invalid_count() == 3
        ix.save(tmp_path / "light.ix")
        info = ix.info()
    with R.RMQIndex.load(dA, tmp_path / "light.ix") as ix2:
        assert ix2.info() == info
        v2, i2 = ix2.query(dQ)
        np.testing.assert_array_equal(i2.cpu().numpy(), ei)
        np.testing.assert_array_equal(v2.cpu().numpy().view(np.uint32), v.cpu().numpy().view(np.uint32))
    for bs, micro in ((100, True), (32, True), (1024, False)):
        with pytest.raises(R.RMQError):
            R.RMQIndex(dA, bs, light=True, micro=micro)


@pytest.mark.parametrize("bs,lr", [(1 << 10, -3), (1 << 12, -2), (1 << 15, -1)])
def test_light_query_stats(cuda, native, bs, lr):
    """The counting kernel on a light index: no per-element entries are
    read; the open queries scan value lines instead."""
    import torch

    import rtxrmq_gb300 as R
    n, q = (1 << 22) + 77, 1 << 16
    A = R.gen_values_uniform(n, 31)
    Q = R.gen_queries(q, n, lr, 32)
    with R.RMQIndex(torch.from_numpy(A).to(cuda), bs, light=True) as ix:
        st = ix.query_stats(torch.from_numpy(Q).to(cuda))
    assert st["entries"] == 0
    settled = sum(st[k] for k in ("first_probe", "second_probe", "full", "micro_scan", "invalid"))
    assert settled == q
    if st["second_probe"] + st["full"]:
        assert st["scan_sectors"] > st["micro_scan"]


def key_order(bits, op):
    """The engine's order of float32 values (as uint32 bits): -0 == +0, NaN
    (quiet or signaling, either sign) after every number; for op "max" the
    reverse of the numbers, NaN still last."""
    b = bits.astype(np.uint32)
    a = b & np.uint32(0x7fffffff)
    k = np.where(b >> 31 == 1, ~b, b | np.uint32(0x80000000)).astype(np.uint32)
    k[a == 0] = np.uint32(0x80000000)
    nan = a > np.uint32(0x7f800000)
    if op == "max":
        k = ~k
    k[nan] = np.uint32(0xffffffff)
    return k


def nan_case(seed, n):
    """float32 values with quiet and signaling NaNs of both signs, +-0 and
    +-inf among normal values, and queries of every length class."""
    import rtxrmq_gb300 as R
    rng = np.random.default_rng(seed)
    A = rng.standard_normal(n).astype(np.float32)
    bits = A.view(np.uint32)
    for pattern, cnt in ((0x7fc00000, n // 40), (0xffc00000, n // 40), (0x7f800001, n // 40),
                         (0xffbfffff, n // 40), (0x00000000, n // 30), (0x80000000, n // 30),
                         (0x7f800000, 20), (0xff800000, 20)):
        bits[rng.integers(0, n, cnt)] = pattern
    # runs of NaN only, so that some queries see nothing else
    for s in rng.integers(0, n - 100, 10):
        bits[s:s + int(rng.integers(1, 90))] = rng.choice([0x7fc00000, 0xffbfffff, 0x7f800001])
    Q = np.concatenate([R.gen_queries(4000, n, L, seed + L) for L in (1, 2, 5, 33, 300, 3000)])
    return A, Q


def expect_nan_case(A, Q, op):
    k = key_order(A.view(np.uint32), op)
    ei = np.array([l + int(np.argmin(k[l:r + 1])) for l, r in Q], dtype=np.int32)
    ev = np.where(k[ei] == np.uint32(0xffffffff), np.uint32(0x7fc00000), A.view(np.uint32)[ei])
    return ei, ev


@pytest.mark.parametrize("op", ["min", "max"])
@pytest.mark.parametrize("light", [False, True])
def test_nan_and_signed_zero_order(cuda, native, op, light):
    """NaNs (quiet and signaling, both signs) order after every number and
    come back as the canonical quiet NaN; +-0 are equal (leftmost wins, its
    own sign returned). Full and light index, both float modes, block sizes
    across the micro-block and block paths; the light index's micro-block
    minima take each lane's IEEE minimum, which must skip every NaN."""
    n = 6007
    A, Q = nan_case(11 + light, n)
    ei, ev = expect_nan_case(A, Q, op)
    for bs in (64, 256, 2048):
        v, i, _ = run_light(cuda, A, Q, bs, op=op) if light else run_full(cuda, A, Q, bs, op)
        np.testing.assert_array_equal(i, ei)
        np.testing.assert_array_equal(v.view(np.uint32), ev)


def run_full(cuda, A, Q, bs, op):
    import torch

    import rtxrmq_gb300 as R
    with R.RMQIndex(torch.from_numpy(A).to(cuda), bs, op=op) as ix:
        v, i = ix.query(torch.from_numpy(np.ascontiguousarray(Q, dtype=np.int32)).to(cuda))
        torch.cuda.synchronize()
        return v.cpu().numpy(), i.cpu().numpy(), None
