"""The bench's replica path on CPU: two gloo ranks (world size 2).

One process per GPU runs an independent product; the job's time is the
slowest rank's (a MAX all-reduce) and its value is every rank's output limbs
over that time.  No collective touches the data path.  Here each rank
multiplies its own seeded operands with the CPU oracle, the ranks agree on
the reduced time, and the products differ between ranks.
"""

import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, q):
    import sys

    import torch.distributed as dist

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "oracle")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=2)
    try:
        import bench
        import oracle as O

        from hypergeometrica_gb300 import workloads as W

        sx, sy = bench.rank_seeds(rank)
        x, y = W.limbs(sx, 64), W.limbs(sy, 64)
        prod = O.mpz_mul_ntt(x, y)[:128]
        ms = bench.max_over_ranks(10.0 + rank, dist, "cpu")
        rate = bench.job_rate(2, 128, 5, ms / 1000.0)
        q.put((rank, ms, rate, bytes(prod.tobytes())))
    finally:
        dist.destroy_process_group()


def test_two_rank_replicas(oracle):
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    assert [r[1] for r in res] == [11.0, 11.0]  # both ranks report the slowest time
    assert res[0][2] == res[1][2] == pytest.approx(2 * 128 * 5 / 0.011)
    assert res[0][3] != res[1][3]  # independent replicas: different operands
    import bench

    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.rank_seeds(0) != bench.rank_seeds(1)
