"""Several GPUs (one process each): events are independent, so ranks take
disjoint event-id ranges -- the Philox streams are keyed by the global event
id, so every event is the same whichever rank computes it -- and nothing is
exchanged on the data path.  The one reduction is the merge of averaged
profiles (event means of several ranks into one), done once at the end.

Works with any torch.distributed backend (NCCL between GPUs, gloo on the
host); host numpy arrays are reduced as CPU tensors, so use a gloo group for
them when the default group is NCCL.
"""
from __future__ import annotations

import numpy as np
import torch
import torch.distributed as dist


def event_range(first_event: int, n_total: int, rank: int, world: int) -> tuple[int, int]:
    """(first, n) of rank's contiguous share of events [first_event,
    first_event + n_total): the first n_total % world ranks take one more."""
    base, extra = divmod(n_total, world)
    n = base + (1 if rank < extra else 0)
    first = first_event + rank * base + min(rank, extra)
    return first, n


def step_events(step: int, rank: int, world: int, n: int) -> int:
    """First event id of rank's batch of n events in a sequence of steps
    (batch k of rank r is the (k * world + r)-th block of n ids)."""
    return (step * world + rank) * n


def merge_means(mean: np.ndarray, count, group=None) -> tuple[np.ndarray, np.ndarray]:
    """Event means of every rank merged into the mean over all ranks'
    events: sum_r count_r mean_r / sum_r count_r, per leading index when
    count is an array (Npart bins) or for the whole array when it is a
    number.  Returns (merged mean, total count) on every rank."""
    m = np.ascontiguousarray(mean, dtype=np.float64)
    c = np.atleast_1d(np.asarray(count, dtype=np.float64))
    w = c.reshape(c.shape + (1,) * (m.ndim - c.ndim)) if c.size > 1 else c[0]
    s = torch.from_numpy(m * w)
    t = torch.from_numpy(c.copy())
    dist.all_reduce(s, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    tot = t.numpy()
    wt = tot.reshape(tot.shape + (1,) * (m.ndim - tot.ndim)) if tot.size > 1 else tot[0]
    with np.errstate(invalid="ignore", divide="ignore"):
        merged = np.where(wt > 0, s.numpy() / np.where(wt > 0, wt, 1), 0.0)
    return merged, tot if tot.size > 1 else tot[0]


def max_over_ranks(x: float, group=None) -> float:
    """The largest value over the ranks (the slowest rank's time)."""
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())
