"""Sharding of independent field lines across ranks (one GPU per rank).

Lines never interact, so the path shards by contiguous line ranges with no
exchange during tracing; results are gathered only if the caller wants them
in one place, and the adjoint's charge gradients are summed with one
all-reduce.  The reference's multi-device split
(GPGPU_Segment/src/CL_Electrostatics.cpp:113-183) sizes shares by compute
units; here ranks are identical GPUs, so shares differ by at most one line.
"""
import numpy as np


def shard_range(n, world, rank):
    """Contiguous [begin, end) of n lines for `rank` of `world`."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world/rank")
    base, extra = divmod(n, world)
    begin = rank * base + min(rank, extra)
    return begin, begin + base + (1 if rank < extra else 0)


def gather_lines(local, n, world, rank, group=None):
    """All ranks receive the full (n, ...) array from each rank's shard
    (torch.distributed all_gather over padded shards)."""
    import torch
    import torch.distributed as dist
    b, e = shard_range(n, world, rank)
    width = (n + world - 1) // world
    t = torch.as_tensor(np.asarray(local))
    pad = torch.zeros((width,) + tuple(t.shape[1:]), dtype=t.dtype)
    pad[: e - b] = t
    parts = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    out = []
    for r in range(world):
        rb, re_ = shard_range(n, world, r)
        out.append(parts[r][: re_ - rb])
    return torch.cat(out).numpy()


def adjoint_sharded(grad_fn, seeds, targets, world, rank, group=None):
    """Loss and charge gradients over lines sharded across ranks.

    The loss is a sum over lines and the gradient with respect to the
    charges is a sum of per-line terms, so each rank runs the adjoint on its
    contiguous range of lines and one all-reduce (sum) of the loss and the
    4p gradient entries completes it — the only exchange of the path.
    grad_fn(seeds_shard, targets_shard) -> (loss, grad (p, 4)) runs one
    shard (em.adjoint on this rank's GPU); targets are (3, rows, n).
    Returns (loss, grad) identical on every rank."""
    import torch
    import torch.distributed as dist
    n = len(seeds)
    b, e = shard_range(n, world, rank)
    loss, grad = grad_fn(seeds[b:e], targets[:, :, b:e])
    buf = torch.zeros(1 + np.asarray(grad).size, dtype=torch.float64)
    buf[0] = float(loss)
    buf[1:] = torch.as_tensor(np.asarray(grad, np.float64).ravel())
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    out = buf.numpy()
    return float(out[0]), out[1:].reshape(np.shape(grad))
