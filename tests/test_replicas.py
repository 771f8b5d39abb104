"""The N>1 path (replicas, one process per GPU): per-rank query seeds,
max-over-ranks step time and the whole-job rate, run as two gloo ranks on
the CPU (the same host logic bench.py uses under torchrun with NCCL)."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    from rtxrmq_gb300 import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        assert replicas.world() == (rank, world)
        ms = 2.0 + rank  # rank 1 is the slow replica
        worst = replicas.max_over_ranks(ms)
        out.put((rank, worst, replicas.rank_seed(1321, rank, -1),
                 replicas.job_rate(1 << 26, world, worst)))
    finally:
        dist.destroy_process_group()


def test_replicas_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [3.0, 3.0]            # both see the slowest rank's time
    assert res[0][2] != res[1][2]                          # each replica answers its own queries
    assert res[0][3] == pytest.approx(2 * (1 << 26) / 3e-3)  # all ranks' queries / max time


def test_single_process_is_identity():
    from rtxrmq_gb300 import replicas
    assert replicas.world() == (0, 1)
    assert replicas.max_over_ranks(1.5) == 1.5
    assert replicas.job_rate(1000, 1, 2.0) == pytest.approx(5e5)
    seeds = {replicas.rank_seed(1321, r, lr) for r in range(4) for lr in (-1, -2, -3, 1024)}
    assert len(seeds) == 16


def test_rank_query_sets_differ(native):
    import numpy as np

    import rtxrmq_gb300 as R
    from rtxrmq_gb300 import replicas
    a = R.gen_queries(1000, 10**6, -1, replicas.rank_seed(1321, 0, -1))
    b = R.gen_queries(1000, 10**6, -1, replicas.rank_seed(1321, 1, -1))
    assert not np.array_equal(a, b)
