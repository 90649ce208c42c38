"""Several GPUs, one process each: replicas only.

The sweep path does not exchange data between lattices, so N GPUs run N
disjoint sets of replicas (temperatures, seeds or field values), with no
collective in the hot loop.  What crosses ranks is host-side bookkeeping:

  shard(n, world, rank)       the contiguous block of the n replicas a rank owns
  max_over_ranks(x)           the slowest rank's time (whole-job throughput is
                              the units all ranks processed over that time)
  po_row(T, stats, P)         one replica's po.dat row from its running sums
                              (src/evolve_thermal.cpp:78-86)
  combine_rows(rows)          the law-of-total-variance combination of
                              average_replicas.py:74-103 over rows
  combine_across_ranks(rows)  the same over every rank's rows (all_gather of the
                              rows, then combine_rows on each rank)

Works with any torch.distributed backend (NCCL on the GPUs, gloo on CPU).
"""
from __future__ import annotations

from typing import List, Optional, Sequence

import numpy as np


def shard(n: int, world: int, rank: int) -> range:
    """Replica indices [start, stop) of `rank` when n replicas are split over
    `world` ranks as evenly as possible (the first n % world ranks get one
    more)."""
    if world < 1 or not 0 <= rank < world or n < 0:
        raise ValueError(f"bad shard request n={n} world={world} rank={rank}")
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def max_over_ranks(x: float, group=None) -> float:
    dist = _dist()
    if dist is None:
        return float(x)
    import torch
    dev = "cuda" if dist.get_backend(group) == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())


def po_row(T: float, stats: Sequence[float], P: Optional[float] = None) -> List[float]:
    """T, S, varS, E, varE (and P for Pear) of one replica from mcx_get_stats
    sums (N, sum S, sum S^2, sum E, sum E^2, ...)."""
    n = stats[0]
    if n <= 0:
        raise ValueError("replica without measured sweeps")
    S1, S2, E, E2 = stats[1] / n, stats[2] / n, stats[3] / n, stats[4] / n
    row = [float(T), S1, S2 - S1 * S1, E, E2 - E * E]
    if P is not None:
        row.append(float(P))
    return row


def combine_rows(rows: Sequence[Sequence[float]]) -> List[float]:
    """One combined row: mean T, mean S, mean(varS) + var(S) (ddof 0), the
    same for E, and mean P when every row has it.  Temperatures more than
    1e-3 apart, or rows of different lengths, are an error."""
    if not rows:
        raise ValueError("no rows to combine")
    ncols = len(rows[0])
    if any(len(r) != ncols for r in rows):
        raise ValueError("rows with different column counts")
    a = np.asarray(rows, dtype=np.float64)
    if a[:, 0].max() - a[:, 0].min() > 1e-3:
        raise ValueError("temperatures differ by more than 1e-3")
    out = [a[:, 0].mean(), a[:, 1].mean(), a[:, 2].mean() + a[:, 1].var(ddof=0), a[:, 3].mean(),
           a[:, 4].mean() + a[:, 3].var(ddof=0)]
    if ncols >= 6:
        out.append(a[:, 5].mean())
    return [float(v) for v in out]


def combine_across_ranks(rows: Sequence[Sequence[float]], group=None) -> List[float]:
    """combine_rows over the rows of every rank, in rank order (every rank
    gets the same result)."""
    dist = _dist()
    if dist is None:
        return combine_rows(rows)
    gathered = [None] * dist.get_world_size(group)
    dist.all_gather_object(gathered, [list(map(float, r)) for r in rows], group=group)
    return combine_rows([r for part in gathered for r in part])
