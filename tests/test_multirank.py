"""The N > 1 path on CPU, with gloo ranks in spawned processes.

- bench.py reports the whole job at the slowest rank's step time.
- Instances shard by contiguous ranges (vectorizedadjoint_gb300/shard.py):
  two ranks, each solving its own range with the oracle, gather the same
  gradients bit for bit as one process solving the whole batch.
- The shared-matrix GLV's dA (gradient of the summed cost over every
  instance) is the one cross-rank exchange: its fixed-order sum of block
  partials gives the single-process bits on every rank.
"""
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


def _shard_rank(rank, world, port, q):
    import numpy as np
    import torch
    import torch.distributed as dist

    from oracle import oracle_py as O
    from vectorizedadjoint_gb300 import shard
    from vectorizedadjoint_gb300 import workloads as W
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    # per-instance gradients of a rank's contiguous range, gathered in rank order
    B = 48
    w = W.make("dho", batch=B)
    c = w["cfg"]
    pb = O.problem(c["model"], c["tableau"], c["n"], c["npar"], c["tol"], c["tol"])
    lo, hi = shard.shard_range(B, rank, world)
    r = O.gradient_batch(pb, c["cost"], w["y0"][lo:hi], w["params"][lo:hi], w["t0"][lo:hi], w["t1"][lo:hi])
    mine = np.concatenate([r["dy0"], r["dp"], r["n_acc"][:, None].astype(np.float64)], 1)
    parts = [None] * world
    dist.all_gather_object(parts, (lo, hi, mine))
    grads = np.concatenate([p[2] for p in sorted(parts, key=lambda p: p[0])], 0)
    # shared-matrix GLV: dA of the summed cost, block partials summed in order
    N, BA, block = 6, 22, 4
    rng = np.random.Generator(np.random.PCG64(7))
    A = rng.normal(0.0, 0.2, (N, N))
    A[np.arange(N), np.arange(N)] = -1.0
    rr = rng.uniform(0.5, 1.5, (BA, N))
    x0 = rng.uniform(0.1, 1.0, (BA, N))
    pg = O.problem("glv", "dopri5", N, N + N * N, 1e-7, 1e-7)
    lo, hi = shard.shard_range(BA, rank, world, block)
    dA_inst = [O.gradient(pg, "sum", x0[b], np.concatenate([rr[b], A.ravel()]), 0.0, 5.0)["dp"][N:]
               for b in range(lo, hi)]
    dA = shard.allreduce_fixed_order(shard.block_partials(dA_inst, lo, hi, block), dist)
    q.put((rank, grads, dA))
    dist.destroy_process_group()


def test_sharded_gradients_and_fixed_order_dA(oracle):
    """Two gloo ranks against one process: per-instance gradients and the
    shared dA bit for bit."""
    import numpy as np

    from vectorizedadjoint_gb300 import shard
    from vectorizedadjoint_gb300 import workloads as W
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_shard_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=300) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # single process
    B = 48
    w = W.make("dho", batch=B)
    c = w["cfg"]
    pb = oracle.problem(c["model"], c["tableau"], c["n"], c["npar"], c["tol"], c["tol"])
    r = oracle.gradient_batch(pb, c["cost"], w["y0"], w["params"], w["t0"], w["t1"])
    ref = np.concatenate([r["dy0"], r["dp"], r["n_acc"][:, None].astype(np.float64)], 1)
    N, BA, block = 6, 22, 4
    rng = np.random.Generator(np.random.PCG64(7))
    A = rng.normal(0.0, 0.2, (N, N))
    A[np.arange(N), np.arange(N)] = -1.0
    rr = rng.uniform(0.5, 1.5, (BA, N))
    x0 = rng.uniform(0.1, 1.0, (BA, N))
    pg = oracle.problem("glv", "dopri5", N, N + N * N, 1e-7, 1e-7)
    dA_inst = [oracle.gradient(pg, "sum", x0[b], np.concatenate([rr[b], A.ravel()]), 0.0, 5.0)["dp"][N:]
               for b in range(BA)]
    dA_ref = shard.sum_in_order(shard.block_partials(dA_inst, 0, BA, block))
    for rank, grads, dA in out:
        np.testing.assert_array_equal(grads, ref)
        np.testing.assert_array_equal(dA, dA_ref)
    # the block sum is close to the plain instance-order sum (another order)
    np.testing.assert_allclose(dA_ref, np.sum(dA_inst, 0), rtol=1e-12, atol=1e-15)


def test_shard_ranges_cover_the_batch():
    from vectorizedadjoint_gb300 import shard
    for total, world, block in [(10, 3, 1), (262144, 8, 1), (22, 2, 4), (5, 4, 2), (1, 2, 1)]:
        ranges = [shard.shard_range(total, r, world, block) for r in range(world)]
        assert ranges[0][0] == 0 and ranges[-1][1] == total
        for (a, b), (c, d) in zip(ranges, ranges[1:]):
            assert b == c
        assert all(lo % block == 0 for lo, hi in ranges if hi > lo)
