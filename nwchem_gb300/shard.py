"""Tuple sharding across GPUs (one process per GPU).

The reference hands tuples to ranks through a Global Arrays shared counter
(nxtask, src/util/nxtask.F:23-80) and sums the two energies with
ga_dgop(1975, energy, 2, '+') (src/tce/ccsd_t/ccsd_t.F:296-297).  Here each
rank takes a fixed, disjoint set of tuples (round-robin over the
weight-ordered list, so every rank gets a similar mix of sizes); there is no
collective on the data path.  The per-rank (E[T], E(T)) pairs are combined
with math.fsum, which is exactly rounded, so the total does not depend on
the number of ranks or on the order in which partials arrive.
"""
from __future__ import annotations

import math
from typing import Iterable, Sequence

import numpy as np


def rank_tasks(n_tasks: int, world: int, rank: int) -> np.ndarray:
    """Indices of the tuples rank `rank` of `world` evaluates."""
    if not (0 <= rank < world):
        raise ValueError("rank out of range")
    return np.arange(rank, n_tasks, world, dtype=np.int64)


def combine(partials: Iterable[Sequence[float]]) -> tuple[float, float]:
    """Exactly rounded sum of (E[T], E(T)) pairs."""
    ps = [tuple(p) for p in partials]
    return math.fsum(p[0] for p in ps), math.fsum(p[1] for p in ps)


def allreduce_energies(per_task: np.ndarray, group=None) -> tuple[float, float]:
    """Gathers every rank's per-tuple (E[T], E(T)) rows (torch.distributed,
    any backend) and returns their exactly rounded totals on all ranks."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    local = torch.as_tensor(np.ascontiguousarray(per_task, dtype=np.float64).reshape(-1, 2))
    n = torch.tensor([local.shape[0]], dtype=torch.int64)
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, n, group=group)
    mx = int(max(int(s) for s in sizes))
    pad = torch.zeros((mx, 2), dtype=torch.float64)
    pad[:local.shape[0]] = local
    bufs = [torch.zeros((mx, 2), dtype=torch.float64) for _ in range(world)]
    dist.all_gather(bufs, pad, group=group)
    rows = [b[:int(s)].numpy() for b, s in zip(bufs, sizes)]
    return combine(np.concatenate(rows, axis=0))
