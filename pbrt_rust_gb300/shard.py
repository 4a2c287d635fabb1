"""Splitting the hot path across devices or processes.

Rays and render tasks are independent (SamplerRenderer::run_task,
src/sampler_renderer.rs:61-144, shares nothing between tasks; a ray query
reads only the BVH), so a job shards into contiguous ranges, one per rank,
with the BVH replicated on every rank and no exchange during the work.  The
results merge on the host side:

  * ray batches: rank r traces rays [lo_r, hi_r); the hits concatenate in
    rank order (``gather_rows``);
  * frames: rank r renders tasks [lo_r, hi_r) (``pbrtgpu_render_tasks``);
    every pixel belongs to one task and comes out +0 on the other ranks, so
    the images add up (``sum_images``) to the single-device frame bit for bit.

The merge uses ``torch.distributed`` collectives on whatever backend the
process group has (gloo on the host, nccl on devices).
"""
from __future__ import annotations


def shard_range(n: int, world: int, rank: int) -> tuple[int, int]:
    """Contiguous range of `n` units for `rank` of `world`: sizes differ by at
    most one, earlier ranks take the larger shares."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    if n < 0:
        raise ValueError("n must be >= 0")
    q, r = divmod(n, world)
    lo = rank * q + min(rank, r)
    return lo, lo + q + (1 if rank < r else 0)


def task_range(num_tasks: int, world: int, rank: int) -> tuple[int, int]:
    """The render tasks of one rank (tasks are the reference's units of work,
    sampler_renderer.rs:39-75)."""
    return shard_range(num_tasks, world, rank)


def gather_rows(local, n_total: int, group=None):
    """Concatenates every rank's rows (the rank-order shards of `n_total`
    rows) on every rank; `local` is a tensor whose first dimension is this
    rank's share."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    lo, hi = shard_range(n_total, world, rank)
    if local.shape[0] != hi - lo:
        raise ValueError(f"rank {rank} holds {local.shape[0]} rows, its shard has {hi - lo}")
    width = shard_range(n_total, world, 0)[1]  # the largest share
    pad = torch.zeros((width,) + tuple(local.shape[1:]), dtype=local.dtype, device=local.device)
    pad[: hi - lo] = local
    parts = [torch.empty_like(pad) for _ in range(world)]
    dist.all_gather(parts, pad, group=group)
    rows = []
    for r in range(world):
        a, b = shard_range(n_total, world, r)
        rows.append(parts[r][: b - a])
    return torch.cat(rows, 0)


def sum_images(img, group=None):
    """Adds the shard images of every rank in place (each pixel is nonzero on
    one rank at most, so the sum is exact)."""
    import torch.distributed as dist
    dist.all_reduce(img, op=dist.ReduceOp.SUM, group=group)
    return img
