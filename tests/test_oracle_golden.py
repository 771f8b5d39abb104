"""CPU: pin the oracle against the reference's own outputs.

The golden vectors under tests/golden/ were produced by the reference's
cpu_rmq / cpu_rmq_idx / rmq_rmm_par(_idx) compiled unmodified
(tests/golden/make_golden.py). The oracle's restatements must reproduce
them exactly; where the reference tree is present the same comparison also
runs live on fresh random inputs.
"""
from pathlib import Path

import numpy as np
import pytest

GOLDEN = sorted((Path(__file__).parent / "golden").glob("*.npz"))


def bits(x):
    return np.ascontiguousarray(x, dtype=np.float32).view(np.uint32)


def test_golden_present():
    assert len(GOLDEN) >= 9


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: p.stem)
def test_base_restatement_matches_reference(path, oracle_lib):
    g = np.load(path)
    A, Q = g["A"], g["Q"]
    np.testing.assert_array_equal(oracle_lib.base_idx(A, Q), g["base_idx"])
    np.testing.assert_array_equal(bits(oracle_lib.base_val(A, Q)), bits(g["base_val"]))


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: p.stem)
@pytest.mark.parametrize("bs", [1, 3, 32, 100, 1024, 1 << 15])
def test_blocks_restatement_matches_reference(path, bs, oracle_lib):
    g = np.load(path)
    A, Q = g["A"], g["Q"]
    v, i = oracle_lib.Blocks(A, bs).query(Q)
    np.testing.assert_array_equal(i, g["base_idx"])
    np.testing.assert_array_equal(bits(v), bits(g["base_val"]))


@pytest.mark.parametrize("path", [p for p in GOLDEN if p.stem != "special_values"],
                         ids=lambda p: p.stem)
def test_hrmq_relations(path):
    """HRMQ values equal BASE; HRMQ indices are rightmost on ties and the
    reversed-array adapter gives BASE's leftmost indices."""
    g = np.load(path)
    A, Q = g["A"], g["Q"]
    np.testing.assert_array_equal(bits(g["hrmq_val"]), bits(g["base_val"]))
    np.testing.assert_array_equal(g["hrmq_rev_idx"], g["base_idx"])
    # native HRMQ index: same minimum value, never left of BASE's index
    np.testing.assert_array_equal(bits(A[g["hrmq_idx"]]), bits(g["base_val"]))
    assert (g["hrmq_idx"] >= g["base_idx"]).all()


def test_ties_make_hrmq_differ():
    """On the tie-heavy case HRMQ's native indices differ from leftmost."""
    g = np.load(Path(__file__).parent / "golden" / "ties_int16.npz")
    assert (g["hrmq_idx"] != g["base_idx"]).sum() > 100


def test_live_against_reference(oracle_lib, native):
    if not oracle_lib.ref_available():
        pytest.skip("reference CPU code not built here")
    import rtxrmq_gb300 as R
    for seed in range(3):
        n = 3000 + 517 * seed
        A = R.gen_values_int(n, 7, seed)
        Q = np.concatenate([R.gen_queries(500, n, -1, seed), R.gen_queries(500, n, 5, seed)])
        np.testing.assert_array_equal(oracle_lib.base_idx(A, Q), oracle_lib.ref_cpu_rmq_idx(A, Q))
        v, i = oracle_lib.Blocks(A, 64 + seed).query(Q)
        np.testing.assert_array_equal(i, oracle_lib.ref_cpu_rmq_idx(A, Q))


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: p.stem)
def test_hrmq_port_matches_reference_hrmq(path, oracle_lib):
    """oracle/hrmq_port.c (HRMQ restated) reproduces the reference HRMQ's
    native indices (rightmost on ties) wherever the fixture has them, and
    BASE's leftmost indices and value bits in strict mode."""
    g = np.load(path)
    A, Q = g["A"], g["Q"]
    if "hrmq_idx" in g:
        v, i = oracle_lib.HRMQ(A, strict=False).query(Q)
        np.testing.assert_array_equal(i, g["hrmq_idx"])
        np.testing.assert_array_equal(bits(v), bits(g["hrmq_val"]))
    v, i = oracle_lib.HRMQ(A, strict=True).query(Q)
    np.testing.assert_array_equal(i, g["base_idx"])
    np.testing.assert_array_equal(bits(v), bits(g["base_val"]))


def test_hrmq_port_large_random(oracle_lib, native):
    """n = 2^20 with heavy ties, every length class: strict mode equals the
    block restatement; native mode returns a minimum at or right of it."""
    import rtxrmq_gb300 as R
    n = 1 << 20
    A = R.gen_values_int(n, 64, 17)
    Q = np.concatenate([R.gen_queries(4000, n, L, 3) for L in (-1, -2, -3, 1, 2, 64, 1000)])
    ev, ei = oracle_lib.Blocks(A, 4096).query(Q)
    v, i = oracle_lib.HRMQ(A, strict=True).query(Q)
    np.testing.assert_array_equal(i, ei)
    v2, i2 = oracle_lib.HRMQ(A, strict=False).query(Q)
    np.testing.assert_array_equal(bits(v2), bits(ev))
    assert (i2 >= ei).all() and (i2 <= Q[:, 1]).all()
