"""Sharding a jagged array over ranks (one GPU per rank).

Lists are independent, so a ListOffsetArray splits into contiguous list
ranges, balanced by lists + elements (the same measure the kernels balance
warps by).  Per shard:

* reductions (sum, max, argmax, count, ...) need no exchange: each rank
  reduces its lists; argmax results are global element indices, so a rank
  adds its shard's first element;
* operations that produce new offsets (jagged getitem, combinations, range
  slices) compute local offsets from 0 and rebase them by the exclusive
  prefix of the per-shard totals -- one allgather of one int64 per rank, the
  only collective.

The functions take numpy arrays (host side) or torch tensors; the rebasing
uses torch.distributed when a process group is initialised.
"""

from __future__ import annotations

import numpy as np


def shard_bounds(offsets, world):
    """List boundaries [l_0 = 0, l_1, ..., l_world = nlists] balanced by lists + elements."""
    offsets = np.asarray(offsets)
    n = len(offsets) - 1
    e0 = int(offsets[0]) if n >= 0 else 0
    total = n + (int(offsets[-1]) - e0 if n >= 0 else 0)
    # item position of list l's start: l + offsets[l] - e0 (monotone in l)
    pos = np.arange(n + 1, dtype=np.int64) + (offsets - e0)
    targets = (total * np.arange(1, world, dtype=np.int64)) // world
    cuts = np.searchsorted(pos, targets, side="left")
    return np.concatenate([[0], np.minimum(cuts, n), [n]]).astype(np.int64)


def local_shard(offsets, content, rank, world):
    """(offsets rebased to 0, content slice, first list, first element) of one rank."""
    offsets = np.asarray(offsets)
    b = shard_bounds(offsets, world)
    l0, l1 = int(b[rank]), int(b[rank + 1])
    a, z = int(offsets[l0]), int(offsets[l1])
    return offsets[l0:l1 + 1] - a, content[a:z], l0, a


def exclusive_prefix_of_totals(total, group=None):
    """Sum of the totals of all lower ranks (allgather of one int64).

    The exchanged tensor lives where the group's backend wants it: on the
    rank's current CUDA device for NCCL (which takes no host tensors), in host
    memory for gloo.
    """
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized():
        return 0
    dev = torch.device("cpu")
    if dist.get_backend(group) == "nccl":
        dev = torch.device("cuda", torch.cuda.current_device())
    t = torch.tensor([int(total)], dtype=torch.int64, device=dev)
    world = dist.get_world_size(group)
    parts = [torch.zeros(1, dtype=torch.int64, device=dev) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    rank = dist.get_rank(group)
    return int(sum(int(p.item()) for p in parts[:rank]))


def rebase_offsets(local_offsets, group=None):
    """Local offsets from 0 -> global offsets (exclusive prefix of shard totals added)."""
    local_offsets = np.asarray(local_offsets)
    total = int(local_offsets[-1]) if len(local_offsets) else 0
    return local_offsets + exclusive_prefix_of_totals(total, group)
