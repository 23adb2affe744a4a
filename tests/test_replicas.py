"""Multi-GPU path of bench.py (replicas only) on CPU: two gloo ranks agree on
the slowest rank's time and on the whole-job throughput."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = 100.0 + 50.0 * rank          # rank 1 is the slow one
        slow = bench.slowest_rank_ms(ms, world)
        dist.barrier()
        q.put((rank, slow, bench.replica_throughput(1000, slow, world)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas_agree_on_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert [r[1] for r in res] == [150.0, 150.0]
    assert res[0][2] == pytest.approx(2 * 1000 / 0.150)


def test_single_rank_is_unchanged():
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    assert bench.slowest_rank_ms(12.5, 1) == 12.5
    assert bench.replica_throughput(500, 250.0, 1) == pytest.approx(2000.0)
