"""The N > 1 path on CPU: bench.py runs independent replicas per rank (the
instances shard with no data exchange) and reports the whole job at the
slowest rank's step time.  Two gloo ranks check that reduction."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, ms_by_rank, q):
    import torch
    import torch.distributed as dist

    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(ms_by_rank[rank], world, dist, torch)
    q.put((rank, ms, bench.replica_throughput(1000, ms, world)))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    ms_by_rank = [12.5, 20.0]
    procs = [ctx.Process(target=_rank, args=(r, world, port, ms_by_rank, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [20.0, 20.0]
    assert out[0][2] == pytest.approx(2 * 1000 / 0.020)


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(3.0, 1, None, None) == 3.0
    assert bench.replica_throughput(10, 5.0, 1) == pytest.approx(2000.0)
