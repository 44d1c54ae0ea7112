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


def _comm_device(group):
    """The device collectives of `group` run on: the current CUDA device
    for NCCL, the host for gloo."""
    import torch
    import torch.distributed as dist
    if dist.get_backend(group) == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def gather_lines(local, n, world, rank, group=None, axis=0):
    """All ranks receive the full array from each rank's shard of n lines
    along `axis` (torch.distributed all_gather over padded shards).

    `local` is a numpy array or a torch tensor; the exchange runs on the
    group's device (CUDA tensors for NCCL, host tensors for gloo) and the
    result comes back as the input's kind (numpy, or a tensor on the input's
    device)."""
    import torch
    import torch.distributed as dist
    is_np = not isinstance(local, torch.Tensor)
    t = torch.as_tensor(np.asarray(local)) if is_np else local
    home = t.device
    comm = _comm_device(group)
    t = t.to(comm).movedim(axis, 0)
    b, e = shard_range(n, world, rank)
    if t.shape[0] != e - b:
        raise ValueError(f"rank {rank} holds {t.shape[0]} lines, its shard is {e - b}")
    width = (n + world - 1) // world
    pad = torch.zeros((width,) + tuple(t.shape[1:]), dtype=t.dtype, device=comm)
    pad[: e - b] = t
    parts = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    out = []
    for r in range(world):
        rb, re_ = shard_range(n, world, r)
        out.append(parts[r][: re_ - rb])
    full = torch.cat(out).movedim(0, axis)
    return full.cpu().numpy() if is_np else full.to(home)


def trace_sharded(trace_fn, seeds, world, rank, group=None, gather=True):
    """Strong-scaling split of one trace: rank r traces the contiguous shard
    of lines shard_range(n, world, r) with trace_fn(seeds_shard) -> vertices
    (3, rows, m) and, if asked, all ranks receive the (3, rows, n) result.
    Lines never interact, so tracing needs no exchange; only the optional
    gather communicates.  Returns (vertices, (begin, end))."""
    n = len(seeds)
    b, e = shard_range(n, world, rank)
    v = trace_fn(seeds[b:e])
    if gather:
        v = gather_lines(v, n, world, rank, group=group, axis=2)
    return v, (b, e)


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
    g = torch.as_tensor(np.asarray(grad, np.float64) if not isinstance(grad, torch.Tensor)
                        else grad.double())
    buf = torch.zeros(1 + g.numel(), dtype=torch.float64, device=_comm_device(group))
    buf[0] = float(loss)
    buf[1:] = g.reshape(-1).to(buf.device)
    dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
    out = buf.cpu().numpy()
    return float(out[0]), out[1:].reshape(np.shape(grad))
