"""The multi-replica timing rule of bench.py (max over ranks, whole-job throughput),
run as two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = 100.0 + 50.0 * rank  # rank 1 is the slower replica
    t = bench.max_over_ranks(ms, dist)
    out.put((rank, t))
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_replicas():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(2))
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == {0: 150.0, 1: 150.0}
    # whole-job value: every rank's steps over the slowest rank's time
    steps, world = 10, 2
    assert world * steps / (res[0] / 1e3) == pytest.approx(133.333, rel=1e-4)
