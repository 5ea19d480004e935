"""Replica sharding across GPUs (one process per GPU).

Events are independent: an event reads only its own x row and the read-only channel
programs, so N GPUs run N replicas of the single-GPU path with no exchange on the data
path.  This module holds the host-side bookkeeping:

* ``event_window``: the contiguous slice of a Philox stream a rank generates (Philox is
  counter-based, so rank r's window is the same numbers a single process would draw for
  those events);
* ``channel_shards``: whole channels assigned to ranks for a multi-channel batch, balanced
  by event count (a channel's events stay on one GPU, so each rank keeps the
  one-launch-per-batch form);
* ``max_over_ranks``: the slowest rank's elapsed time (the only collective, outside the
  data path, for timing).
"""
from __future__ import annotations

from typing import List, Tuple

import numpy as np


def event_window(rank: int, world: int, n_total: int) -> Tuple[int, int]:
    """(first event, count) of rank's share of n_total events: contiguous, sizes differ by
    at most one."""
    if not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(int(n_total), int(world))
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def channel_shards(counts, world: int) -> List[np.ndarray]:
    """Channel indices per rank, every channel on exactly one rank, balanced by events
    (largest channels first, each to the currently lightest rank)."""
    counts = np.asarray(counts, np.int64)
    load = np.zeros(world, np.int64)
    owner = np.zeros(len(counts), np.int64)
    for c in np.argsort(-counts, kind="stable"):
        r = int(np.argmin(load))
        owner[c] = r
        load[r] += counts[c]
    return [np.nonzero(owner == r)[0] for r in range(world)]


def max_over_ranks(value: float) -> float:
    """The largest value over the ranks of the default process group (the value itself
    when torch.distributed is not initialised)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
