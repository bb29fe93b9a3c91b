"""Data parallelism over independent systems (one process per GPU).

The reference shards its batch axis with ``shard_map`` and no collectives
(src/kups/application/utils/propagate.py:148-176): systems never exchange
data during a step.  Here each rank takes a contiguous range of whole systems,
chosen so that the ranks' costs (atoms, or atoms squared for the pair work of
dense systems) are as equal as contiguous ranges allow, runs its systems with
the single-GPU kernels, and only per-system observables are gathered to rank 0
for logging (a host-side gather, not part of the step).
"""

from __future__ import annotations

import numpy as np
import torch


def partition_by_cost(costs, world: int) -> list[tuple[int, int]]:
    """Contiguous ranges [lo, hi) of systems, one per rank, minimising the largest range cost.

    Exact for contiguous splits: binary search on the bottleneck cost, greedy packing
    (every range as long as the bound allows) as the feasibility test.
    """
    c = np.asarray(costs, dtype=np.float64)
    if world < 1:
        raise ValueError("world must be >= 1")
    if np.any(c < 0):
        raise ValueError("costs must be non-negative")
    n = len(c)
    prefix = np.concatenate([[0.0], np.cumsum(c)])

    def pack(bound):
        ranges, lo = [], 0
        for _ in range(world):
            # furthest hi with prefix[hi] - prefix[lo] <= bound
            hi = int(np.searchsorted(prefix, prefix[lo] + bound, side="right")) - 1
            hi = max(hi, lo + 1) if lo < n else lo
            hi = min(hi, n)
            ranges.append((lo, hi))
            lo = hi
        return ranges, lo >= n

    lo_b, hi_b = float(c.max(initial=0.0)), float(prefix[-1])
    best, _ = pack(hi_b)
    for _ in range(100):
        if hi_b - lo_b <= 1e-9 * max(1.0, hi_b):
            break
        mid = 0.5 * (lo_b + hi_b)
        r, ok = pack(mid)
        if ok:
            best, hi_b = r, mid
        else:
            lo_b = mid
    r, ok = pack(hi_b)
    if ok:
        best = r
    return best


def rank_systems(n_atoms_per_system, rank: int, world: int, exponent: float = 1.0) -> tuple[int, int]:
    """This rank's system range with cost N_s ** exponent (1: neighbour-list MD, 2: dense pairs)."""
    return partition_by_cost(np.asarray(n_atoms_per_system, np.float64) ** exponent, world)[rank]


def gather_per_system(values: torch.Tensor, ranges, rank: int, group=None) -> torch.Tensor | None:
    """Rank 0 receives the per-system rows of every rank in system order (CPU tensors on
    gloo, device tensors on NCCL); other ranks get None."""
    import torch.distributed as dist

    world = len(ranges)
    counts = [hi - lo for lo, hi in ranges]
    width = max(counts) if counts else 0
    pad = torch.zeros((width,) + tuple(values.shape[1:]), dtype=values.dtype, device=values.device)
    pad[: values.shape[0]] = values
    bufs = [torch.empty_like(pad) for _ in range(world)] if rank == 0 else None
    dist.gather(pad, bufs, dst=0, group=group)
    if rank != 0:
        return None
    return torch.cat([b[:n] for b, n in zip(bufs, counts)])
