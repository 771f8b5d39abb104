"""GPU: rmq_query_noalloc, the build + query entry point that allocates no
device memory (for callers that are not allowed to: a host framework that
owns all device memory through its own pool, or a latency-critical loop that
cannot take cudaMalloc's implicit device-wide synchronisation). Its index
lives in a fixed device array inside librmq.so.

Called through the C ABI and compared with the allocating entry points
(rmq_build + rmq_query) on the same inputs, bit-exact (values and indices),
on two calls in a row with different arrays, block sizes and queries, so a
second call must not see the first call's state. Collected last so that a
run stopping at its first failure has run every other test already; it
also passes on its own in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def reference_path(native, dA, n, bs, dQ, q, cuda):
    """Outputs of the existing entry points: rmq_build + rmq_query."""
    import torch

    from rtxrmq_gb300._native import check
    h = C.c_void_p()
    s = torch.cuda.current_stream().cuda_stream
    check(native.rmq_build(dA.data_ptr(), n, bs, s, C.byref(h)))
    v = torch.empty(q, dtype=torch.float32, device=cuda)
    i = torch.empty(q, dtype=torch.int32, device=cuda)
    check(native.rmq_query(h, dQ.data_ptr(), q, v.data_ptr(), i.data_ptr(), s))
    torch.cuda.synchronize()
    check(native.rmq_free(h))
    return v.cpu().numpy(), i.cpu().numpy()


def test_noalloc_matches_allocating_path(cuda, native):
    import torch

    import rtxrmq_gb300 as R
    from rtxrmq_gb300._native import check
    cases = [
        (1_000_000, 1024, -3, 11),  # first call: sub-block level, short ranges
        (777_777, 1000, -1, 12),    # second call: smaller array, other block size
        # third call: the index fits the scratch only without the sub-block
        # level (4 x 8 MiB of per-element entries alone fill it), so the
        # entry point plans, places and answers from the plain index
        (1 << 20, 64, -2, 13),
    ]
    for n, bs, lr, seed in cases:
        A = R.gen_values_int(n, 1000, seed)  # many ties
        Q = R.gen_queries(300_000, n, lr, seed)
        Q[:3] = [[5, 4], [0, n], [-1, 2]]  # invalid queries: -1 / NaN
        dA = torch.from_numpy(A).to(cuda)
        dQ = torch.from_numpy(Q).to(cuda)
        q = len(Q)
        ev, ei = reference_path(native, dA, n, bs, dQ, q, cuda)
        v = torch.full((q,), 7.0, dtype=torch.float32, device=cuda)
        i = torch.full((q,), -7, dtype=torch.int32, device=cuda)
        s = torch.cuda.current_stream().cuda_stream
        check(native.rmq_query_noalloc(dA.data_ptr(), n, bs, dQ.data_ptr(), q, v.data_ptr(),
                                       i.data_ptr(), s))
        torch.cuda.synchronize()
        np.testing.assert_array_equal(i.cpu().numpy(), ei)
        np.testing.assert_array_equal(v.cpu().numpy().view(np.uint32), ev.view(np.uint32))
        assert list(ei[:3]) == [-1, -1, -1]


def test_noalloc_rejects_oversize(cuda, native):
    """An index larger than the fixed scratch is refused with RMQ_EINVAL."""
    import torch
    dA = torch.zeros(4_000_000, dtype=torch.float32, device=cuda)
    dQ = torch.zeros((1, 2), dtype=torch.int32, device=cuda)
    out = torch.empty(1, dtype=torch.int32, device=cuda)
    rc = native.rmq_query_noalloc(dA.data_ptr(), dA.numel(), 1024, dQ.data_ptr(), 1, None,
                                  out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == -1
    assert b"static scratch" in native.rmq_last_error_string()
