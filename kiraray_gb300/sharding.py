"""Multi-GPU layout of the wavefront pass: replicas.

A frame has no exchange between pixels, so N GPUs each hold a full scene
replica and render a contiguous band of rows (or whole views); the only
collective is the final image gather.  A data-parallel neural radiance cache
would add one gradient all-reduce per training step (`allreduce_mean`).
These helpers are host logic over torch.distributed (NCCL on GPUs, gloo in
the CPU tests).
"""
from __future__ import annotations

import torch
import torch.distributed as dist


def row_band(width: int, height: int, rank: int, world: int) -> tuple[int, int]:
    """Pixel-index range [begin, end) of the rows owned by `rank` (row-major
    pixels; bands differ in size by at most one row)."""
    if not 0 <= rank < world:
        raise ValueError("rank out of range")
    base, extra = divmod(height, world)
    r0 = rank * base + min(rank, extra)
    r1 = r0 + base + (1 if rank < extra else 0)
    return r0 * width, r1 * width


def gather_rows(local: torch.Tensor, width: int, height: int, rank: int, world: int,
                group=None) -> torch.Tensor | None:
    """Gathers each rank's band (float [pixels_of_band, C]) into the full
    image on rank 0 (None elsewhere)."""
    if world == 1:
        return local
    bands = [row_band(width, height, r, world) for r in range(world)]
    longest = max(e - b for b, e in bands)
    pad = torch.zeros((longest, local.shape[1]), dtype=local.dtype, device=local.device)
    pad[: local.shape[0]] = local
    parts = [torch.empty_like(pad) for _ in range(world)] if rank == 0 else None
    dist.gather(pad, parts, dst=0, group=group)
    if rank != 0:
        return None
    return torch.cat([p[: e - b] for p, (b, e) in zip(parts, bands)], 0)


def allreduce_mean(t: torch.Tensor, world: int, group=None) -> torch.Tensor:
    """Mean over ranks (gradient averaging of a data-parallel cache)."""
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
        t /= world
    return t
