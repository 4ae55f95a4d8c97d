"""The replicas path of bench.py on two CPU ranks (gloo): every rank renders the same workload,
the job's time is the slowest rank's, and the reported rate is the aggregate over ranks. The
rendering itself needs a GPU; the reduction and the aggregation are what differ from N = 1."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import sys
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, repo)
    import bench
    ms = 10.0 + 5.0 * rank            # rank 1 is the slower one
    t = bench.max_over_ranks(ms, "cpu")
    rate = bench.aggregate_rate(30, t / 1000.0, world)
    out.put((rank, t, rate))
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank_and_aggregate():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]
    assert res[0][2] == pytest.approx(2 * 30 / 0.015)
    assert res[0][2] == res[1][2]


def test_single_rank_needs_no_process_group():
    import bench
    assert bench.max_over_ranks(12.5, "cpu") == 12.5
    assert bench.aggregate_rate(30, 0.3, 1) == pytest.approx(100.0)
