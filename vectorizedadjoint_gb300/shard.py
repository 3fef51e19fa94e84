"""Instance sharding across processes (one GPU each).

Instances are independent, so a batch shards by contiguous instance ranges
with no exchange on the data path: rank r of W solves instances
[lo_r, hi_r).  The one exchange is the shared-matrix GLV's dA, the gradient
of the summed cost over ALL instances with respect to the common A: each
rank holds the sum over its own instances, and the job's dA is their sum.

That sum is taken in a fixed order that does not depend on the number of
ranks: instances are grouped into blocks of `block` consecutive instances,
each block's partial is the sum of its instances in index order, and dA is
the sum of the block partials in block order.  Ranks own whole blocks
(contiguous block ranges), gather every block partial and add them in block
order, so any world size -- and a single process -- gives the same bits.
"""
import numpy as np


def shard_range(total, rank, world, block=1):
    """Contiguous [lo, hi) instance range of `rank`: whole blocks of `block`
    instances, split as evenly as possible (the last block may be short)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must lie in [0, world)")
    nblocks = -(-total // block)
    per, extra = divmod(nblocks, world)
    b0 = rank * per + min(rank, extra)
    b1 = b0 + per + (1 if rank < extra else 0)
    return min(total, b0 * block), min(total, b1 * block)


def block_partials(per_instance, lo, hi, block):
    """Block partials of instances [lo, hi) (lo on a block boundary):
    per_instance[i - lo] summed in index order within each block.
    Returns an array [nblocks, ...]."""
    if lo % block:
        raise ValueError("a shard starts on a block boundary")
    x = np.asarray(per_instance, dtype=np.float64)
    out = []
    for s in range(0, hi - lo, block):
        acc = np.zeros_like(x[0])
        for i in range(s, min(s + block, hi - lo)):
            acc = acc + x[i]
        out.append(acc)
    return np.stack(out) if out else np.zeros((0,) + x.shape[1:])


def sum_in_order(partials):
    """The fixed-order total of block partials [nblocks, ...] (block order)."""
    acc = np.zeros_like(partials[0])
    for p in partials:
        acc = acc + p
    return acc


def allreduce_fixed_order(local_partials, dist, group=None):
    """Every rank's block partials gathered (torch.distributed all_gather of
    equal-shaped tensors, padded), concatenated in rank order and summed in
    block order: the same bits on every rank, for any world size.
    local_partials: numpy [nblocks_r, ...] (nblocks_r may differ by one)."""
    import torch

    world = dist.get_world_size(group)
    x = torch.from_numpy(np.ascontiguousarray(local_partials, dtype=np.float64))
    n = torch.tensor([x.shape[0]], dtype=torch.int64)
    counts = [torch.zeros_like(n) for _ in range(world)]
    dist.all_gather(counts, n, group=group)
    width = int(max(int(c) for c in counts))
    pad = torch.zeros((width,) + tuple(x.shape[1:]), dtype=torch.float64)
    pad[:x.shape[0]] = x
    bufs = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(bufs, pad, group=group)
    ordered = [bufs[r][:int(counts[r])].numpy() for r in range(world)]
    return sum_in_order(np.concatenate(ordered, axis=0))


def sum_over_ranks_in_order(local, dist, group=None):
    """Sum of one array per rank, added in rank order (rank 0 first) on every
    rank: deterministic for a given world size (torch all_gather)."""
    import torch

    world = dist.get_world_size(group)
    x = torch.as_tensor(np.ascontiguousarray(local, dtype=np.float64))
    bufs = [torch.zeros_like(x) for _ in range(world)]
    dist.all_gather(bufs, x, group=group)
    acc = bufs[0].clone()
    for r in range(1, world):
        acc = acc + bufs[r]
    return acc.numpy()
