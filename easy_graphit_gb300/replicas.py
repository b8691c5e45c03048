"""Multi-GPU execution of independent traversal units (host logic).

A single traversal does not shard -- it would need a frontier exchange every
iteration -- so several GPUs run *replicas*: every rank holds the whole graph
and traverses its own sources (or its own graphs of a multi-graph batch).
There is no collective on the data path; the only cross-rank traffic is the
barrier around the timed region and a max-reduction of the elapsed time.
"""
from __future__ import annotations

from typing import Sequence

import numpy as np

from .graphit import K_RAND_SEED, HostGraph


def rank_sources(hg: HostGraph, n: int, rank: int, seed: int = K_RAND_SEED) -> np.ndarray:
    """Weak scaling: rank r draws its own n sources with SourcePicker seed+r."""
    return hg.pick_sources(n, seed=seed + rank)


def shard(units: Sequence[int], rank: int, world: int) -> list:
    """Strong scaling: contiguous near-equal shards of a global unit list."""
    n = len(units)
    lo = (n * rank) // world
    hi = (n * (rank + 1)) // world
    return list(units[lo:hi])


def max_over_ranks(value: float, device=None) -> float:
    """Max of a per-rank scalar (the elapsed time of the timed region)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def aggregate_teps(local_edges: float, local_ms: float, device=None) -> tuple[float, float]:
    """Whole-job TEPS: edges traversed by all ranks / the slowest rank's time.
    Returns (GTEPS, max ms)."""
    ms = max_over_ranks(local_ms, device)
    edges = sum_over_ranks(local_edges, device)
    return edges / (ms / 1e3) / 1e9, ms
