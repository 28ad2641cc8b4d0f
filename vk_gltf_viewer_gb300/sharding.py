"""View sharding across ranks (one process per GPU).

Views are independent: each rank culls, rasterises and resolves its own
subset with no collective on the data path.  The adjoint adds one exchange,
a sum all-reduce of the position, colour and texel gradients after each
rank's local backward pass.
"""
from __future__ import annotations

import torch


def shard_views(pixel_counts, world: int, rank: int) -> list[int]:
    """Indices of the views rank `rank` renders, balancing pixel counts.

    Longest-processing-time greedy: views sorted by pixel count (descending,
    index as tie-break) are handed one by one to the rank with the fewest
    pixels so far (lowest rank on ties).  Deterministic, so every rank
    computes the same partition without communicating; every view lands on
    exactly one rank.  Returned indices are ascending.
    """
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside world of {world}")
    counts = [int(c) for c in pixel_counts]
    if any(c < 0 for c in counts):
        raise ValueError("pixel counts must be non-negative")
    load = [0] * world
    owner = [0] * len(counts)
    for i in sorted(range(len(counts)), key=lambda k: (-counts[k], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        owner[i] = r
        load[r] += counts[i]
    return [i for i, o in enumerate(owner) if o == rank]


def allreduce_gradients(grads, group=None) -> None:
    """Sums the gradient tensors over all ranks in place with one collective:
    the tensors are packed into one flat buffer, reduced, and unpacked."""
    import torch.distributed as dist

    grads = [g for g in grads if g is not None]
    if not grads:
        return
    dtype, device = grads[0].dtype, grads[0].device
    for g in grads:
        if g.dtype != dtype or g.device != device:
            raise ValueError("gradients must share one dtype and device")
    flat = torch.cat([g.reshape(-1) for g in grads])
    dist.all_reduce(flat, op=dist.ReduceOp.SUM, group=group)
    off = 0
    for g in grads:
        n = g.numel()
        g.copy_(flat[off:off + n].view_as(g))
        off += n
