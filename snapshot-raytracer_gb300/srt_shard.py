"""Pixel-range sharding of the forward and of the vjp across processes (one
GPU each).

Rays are independent, so a sky (or the reference's batch range) splits into
contiguous RING ranges with no communication during the trace; the only
exchange is assembling the maps afterwards, which the reference leaves to the
user (it writes one file per batch, snapshot-raytracer.cu:708-717, :939-987).
The vjp of a loss summed over pixels splits the same way: each rank forms the
gradient of its pixels' share (its slice of the weights) and one sum
all-reduce of the gradient grids gives the full gradient.
"""
import numpy as np


def shard_range(pix_begin, pix_count, rank, world):
    """Contiguous share of [pix_begin, pix_begin + pix_count) for `rank`:
    (begin, count), sizes differing by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world")
    base, extra = divmod(pix_count, world)
    begin = pix_begin + rank * base + min(rank, extra)
    return begin, base + (1 if rank < extra else 0)


def assemble(parts, pix_begin, pix_count, world):
    """Concatenate per-rank (6, count_r) maps in rank order into (6, pix_count)."""
    out = np.zeros((6, pix_count), np.float32)
    for r, part in enumerate(parts):
        b, c = shard_range(pix_begin, pix_count, r, world)
        out[:, b - pix_begin:b - pix_begin + c] = part
    return out


def gather_maps(part, pix_begin, pix_count, group=None):
    """All-gather the ranks' map shards over torch.distributed and assemble
    them (every rank gets the full (6, pix_count) maps)."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    t = torch.from_numpy(np.ascontiguousarray(part, np.float32))
    sizes = [shard_range(pix_begin, pix_count, r, world)[1] for r in range(world)]
    bufs = [torch.zeros((6, s), dtype=torch.float32) for s in sizes]
    if max(sizes) != min(sizes):  # all_gather wants equal sizes: pad to the largest
        m = max(sizes)
        pad = torch.zeros((6, m), dtype=torch.float32)
        pad[:, :t.shape[1]] = t
        full = [torch.zeros((6, m), dtype=torch.float32) for _ in range(world)]
        dist.all_gather(full, pad, group=group)
        bufs = [f[:, :s] for f, s in zip(full, sizes)]
    else:
        dist.all_gather(bufs, t, group=group)
    return assemble([b.numpy() for b in bufs], pix_begin, pix_count, world)


def shard_weights(weights, pix_begin, pix_count, rank, world):
    """The (6, count_r) slice of (6, pix_count) map weights for `rank`'s range,
    with that range: (weights_r, begin_r, count_r)."""
    b, c = shard_range(pix_begin, pix_count, rank, world)
    return np.ascontiguousarray(weights[:, b - pix_begin:b - pix_begin + c]), b, c


def allreduce_gradients(grads, group=None):
    """Sum all-reduce, in place, of the ranks' gradient grids (torch tensors:
    CUDA with NCCL, CPU with gloo; numpy arrays go through a CPU tensor)."""
    import torch
    import torch.distributed as dist

    out = []
    for g in grads:
        if g is None:
            out.append(None)
            continue
        if isinstance(g, np.ndarray):
            t = torch.from_numpy(g)
            dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
            out.append(t.numpy())
        else:
            dist.all_reduce(g, op=dist.ReduceOp.SUM, group=group)
            out.append(g)
    return out
