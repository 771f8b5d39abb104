"""GPU: the differentiable range-min (forward = exact batched min + saved
argmin, backward = hand-written fp32-atomic scatter of grad_out to the argmin).

Tolerances: gradients within 1e-5 relative of an FP64 gather/scatter
reference, relative to the magnitude of what was summed into each element
(sum of |grad_out| over the queries whose argmin it is: the scale of fp32
summation error; where contributions cancel, |g64| alone would be
ill-conditioned), and exactly zero where nothing was scattered; central
finite differences (eps = 1e-3, tie-free rows whose values are >= 1e-2
apart) within 1e-3 relative (float32 rounding of x +- eps).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rows(seed, nrows=24, lmin=200, lmax=5000, qpr=300):
    import rtxrmq_gb300 as R
    rng = np.random.default_rng(seed)
    lens = rng.integers(lmin, lmax, nrows).astype(np.int64)
    n = int(lens.sum())
    x = R.gen_values_normal(n, seed)
    qc = np.full(nrows, qpr, np.int64)
    Q = np.concatenate([R.gen_queries_lognormal(qpr, int(L), 0.4 * np.log(L), 0.5, seed * 100 + i)
                        for i, L in enumerate(lens)])
    return lens, qc, x, Q


def ref_fp64(lens, qc, x, Q, gout, oracle_lib):
    starts = np.concatenate([[0], np.cumsum(lens)[:-1]])
    qs = np.concatenate([[0], np.cumsum(qc)[:-1]])
    val = np.empty(len(Q), np.float32)
    gidx = np.empty(len(Q), np.int64)
    for s, L, a, c in zip(starts, lens, qs, qc):
        q = Q[a:a + c]
        val[a:a + c] = oracle_lib.base_val(x[s:s + L], q)
        gidx[a:a + c] = s + oracle_lib.base_idx(x[s:s + L], q)
    g = np.zeros(len(x), np.float64)
    np.add.at(g, gidx, gout.astype(np.float64))
    scale = np.zeros(len(x), np.float64)
    np.add.at(scale, gidx, np.abs(gout.astype(np.float64)))
    return val, gidx, (g, scale)


def assert_rel(g, ref, tol):
    g64, scale = ref
    hit = scale > 0
    assert np.all(g[~hit] == 0)
    rel = np.abs(g[hit] - g64[hit]) / scale[hit]
    assert rel.max() <= tol, rel.max()


def test_forward_and_fp64_gradient(cuda, native, oracle_lib):
    import torch

    from rtxrmq_gb300.autograd import RaggedRangeMin
    lens, qc, x, Q = rows(1)
    gout = np.random.default_rng(2).standard_normal(len(Q)).astype(np.float32)
    val, gidx, g64 = ref_fp64(lens, qc, x, Q, gout, oracle_lib)
    m = RaggedRangeMin(lens, qc)
    xt = torch.from_numpy(x).to(cuda).requires_grad_(True)
    y, idx = m(xt, torch.from_numpy(Q).to(cuda))
    np.testing.assert_array_equal(y.detach().cpu().numpy().view(np.uint32), val.view(np.uint32))
    starts = np.repeat(np.concatenate([[0], np.cumsum(lens)[:-1]]), qc)
    np.testing.assert_array_equal(idx.cpu().numpy() + starts, gidx)
    y.backward(torch.from_numpy(gout).to(cuda))
    assert_rel(xt.grad.cpu().numpy().astype(np.float64), g64, 1e-5)


def test_finite_differences(cuda, native):
    import torch

    from rtxrmq_gb300.autograd import RaggedRangeMin
    rng = np.random.default_rng(3)
    lens = np.array([60, 97, 41], np.int64)
    n = int(lens.sum())
    x = (rng.permutation(n) * 1e-2 - 1.0).astype(np.float32)  # distinct, >= 1e-2 apart
    qc = np.array([40, 40, 40], np.int64)
    import rtxrmq_gb300 as R
    Q = np.concatenate([R.gen_queries_lognormal(40, int(L), 0.4 * np.log(L), 0.5, 9 + i)
                        for i, L in enumerate(lens)])
    gout = rng.standard_normal(len(Q)).astype(np.float32)
    m = RaggedRangeMin(lens, qc)
    dQ = torch.from_numpy(Q).to(cuda)
    go = torch.from_numpy(gout).to(cuda)
    xt = torch.from_numpy(x).to(cuda).requires_grad_(True)
    y, _ = m(xt, dQ)
    y.backward(go)
    grad = xt.grad.cpu().numpy().astype(np.float64)

    def loss(xv):
        with torch.no_grad():
            yv, _ = m(torch.from_numpy(xv).to(cuda), dQ)
        return float((yv.cpu().numpy().astype(np.float64) * gout.astype(np.float64)).sum())

    eps = 1e-3
    fd = np.empty(n)
    for j in range(n):
        xp, xm = x.copy(), x.copy()
        xp[j] += np.float32(eps)
        xm[j] -= np.float32(eps)
        fd[j] = (loss(xp) - loss(xm)) / (2 * eps)
    assert np.abs(grad).sum() > 0
    nz = np.abs(grad) > 0
    assert np.all(np.abs(fd[~nz]) < 1e-6)
    np.testing.assert_allclose(fd[nz], grad[nz], rtol=1e-3)


def test_graph_captured_step(cuda, native, oracle_lib):
    """Forward + backward captured once in a CUDA graph and replayed."""
    import torch

    from rtxrmq_gb300.autograd import RaggedRangeMin
    lens, qc, x, Q = rows(4, nrows=8)
    gout = np.random.default_rng(5).standard_normal(len(Q)).astype(np.float32)
    m = RaggedRangeMin(lens, qc)
    xt = torch.from_numpy(x).to(cuda).requires_grad_(True)
    dQ = torch.from_numpy(Q).to(cuda)
    go = torch.from_numpy(gout).to(cuda)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(2):
            xt.grad = None
            y, _ = m(xt, dQ)
            y.backward(go)
    torch.cuda.current_stream().wait_stream(s)
    xt.grad = None
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        y, idx = m(xt, dQ)
        y.backward(go)
    for seed in (6, 7):
        import rtxrmq_gb300 as R
        x2 = R.gen_values_normal(len(x), seed)
        with torch.no_grad():
            xt.copy_(torch.from_numpy(x2))
        g.replay()
        torch.cuda.synchronize()
        val, gidx, g64 = ref_fp64(lens, qc, x2, Q, gout, oracle_lib)
        np.testing.assert_array_equal(y.detach().cpu().numpy().view(np.uint32), val.view(np.uint32))
        assert_rel(xt.grad.cpu().numpy().astype(np.float64), g64, 1e-5)


def test_full_size_fp64_gradient(cuda, native, oracle_lib):
    """The differentiable configuration at full size: 256 rows of N(0,1)
    values with lengths uniform in [2^14, 2^20], 2^16 ranges per row
    (2^24 in all, lengths lognormal(0.4 ln len, 0.5)), grad_out N(0,1).
    Forward values and argmins bit-exact against the oracle row by row;
    the gradient within 1e-5 of the FP64 scatter of the same argmins."""
    import torch

    from rtxrmq_gb300 import workloads as W
    from rtxrmq_gb300.autograd import RaggedRangeMin
    d = W.differentiable_rows(nrows=256, q_per_row=1 << 16, seed=1321)
    gout = np.random.default_rng(1321).standard_normal(d.total_q).astype(np.float32)
    m = RaggedRangeMin(d.lengths, d.qcounts)
    xt = torch.from_numpy(d.values).to(cuda).requires_grad_(True)
    y, idx = m(xt, torch.from_numpy(d.queries).to(cuda))
    y.backward(torch.from_numpy(gout).to(cuda))
    torch.cuda.synchronize()
    y = y.detach().cpu().numpy()
    idx = idx.cpu().numpy()
    for s, L, a, c in zip(d.starts, d.lengths, d.qstarts, d.qcounts):
        q = d.queries[a:a + c]
        np.testing.assert_array_equal(idx[a:a + c], oracle_lib.base_idx(d.values[s:s + L], q))
        np.testing.assert_array_equal(y[a:a + c].view(np.uint32),
                                      oracle_lib.base_val(d.values[s:s + L], q).view(np.uint32))
    gidx = idx.astype(np.int64) + np.repeat(d.starts, d.qcounts)
    g64 = np.zeros(d.span, np.float64)
    np.add.at(g64, gidx, gout.astype(np.float64))
    scale = np.zeros(d.span, np.float64)
    np.add.at(scale, gidx, np.abs(gout.astype(np.float64)))
    assert_rel(xt.grad.cpu().numpy().astype(np.float64), (g64, scale), 1e-5)


def test_finite_differences_thousands(cuda, native):
    """Central finite differences (eps = 1e-3) on three tie-free rows of
    ~1000 elements each (values >= 1e-2 apart), every element perturbed:
    the backward's gradient matches within 1e-3 relative, and elements
    that are no query's argmin have zero derivative."""
    import torch

    import rtxrmq_gb300 as R
    from rtxrmq_gb300.autograd import RaggedRangeMin
    rng = np.random.default_rng(11)
    lens = np.array([1000, 1237, 811], np.int64)
    n = int(lens.sum())
    x = (rng.permutation(n) * 1e-2 - 10.0).astype(np.float32)  # distinct, >= 1e-2 apart
    qc = np.array([300, 300, 300], np.int64)
    Q = np.concatenate([R.gen_queries_lognormal(300, int(L), 0.4 * np.log(L), 0.5, 19 + i)
                        for i, L in enumerate(lens)])
    gout = rng.standard_normal(len(Q)).astype(np.float32)
    m = RaggedRangeMin(lens, qc)
    dQ = torch.from_numpy(Q).to(cuda)
    xt = torch.from_numpy(x).to(cuda).requires_grad_(True)
    y, _ = m(xt, dQ)
    y.backward(torch.from_numpy(gout).to(cuda))
    grad = xt.grad.cpu().numpy().astype(np.float64)
    g64 = gout.astype(np.float64)
    xd = torch.from_numpy(x).to(cuda)

    def loss(j, xj):
        with torch.no_grad():
            xd[j] = float(xj)
            yv, _ = m(xd, dQ)
            xd[j] = float(x[j])
        return float((yv.cpu().numpy().astype(np.float64) * g64).sum())

    # divided by the float32 values actually stored, x[j] +- eps rounded
    eps = 1e-3
    fd = np.empty(n)
    for j in range(n):
        xp, xm = np.float32(x[j] + eps), np.float32(x[j] - eps)
        fd[j] = (loss(j, xp) - loss(j, xm)) / (float(xp) - float(xm))
    nz = np.abs(grad) > 0
    assert nz.sum() > 100
    assert np.all(np.abs(fd[~nz]) < 1e-6)
    np.testing.assert_allclose(fd[nz], grad[nz], rtol=1e-3)
