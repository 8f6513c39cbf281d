"""The multi-GPU bench path is replicas (the DM plan does not need an
exchange): ranks time their own search, the job rate is world x units / the
slowest rank's time.  Two gloo ranks on the CPU check the reduction."""
import os
import socket

import pytest


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
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist)
    out.put((rank, ms, bench.replica_throughput(1000.0, ms, world)))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [15.0, 15.0]
    assert got[0][2] == pytest.approx(2 * 1000.0 / 0.015)


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(3.5, None) == 3.5
    assert bench.replica_throughput(100.0, 10.0, 1) == pytest.approx(1e4)
