"""Independent systems shared out over processes, one GPU each.

A single suspension does not split without a halo exchange every step, so
one simulation runs on one GPU and more GPUs run more of them.  An ensemble
of independent systems shards with no data-path collective: the systems are
assigned to ranks by longest-processing-time-first bin packing on their
particle counts (the step cost is linear in particles), each rank steps its
share as one ensemble, and only per-system results travel, gathered once at
the end.
"""
from __future__ import annotations

from typing import Any, Dict, List, Sequence


def lpt_partition(weights: Sequence[float], nranks: int) -> List[List[int]]:
    """Indices of `weights` split into `nranks` groups: heaviest first, each
    onto the currently lightest group (ties to the lower index), so the
    largest group load is at most 4/3 of the optimum (Graham 1969).  Each
    group is returned in increasing index order."""
    if nranks < 1:
        raise ValueError("nranks must be at least 1")
    order = sorted(range(len(weights)), key=lambda i: (-float(weights[i]), i))
    loads = [0.0] * nranks
    parts: List[List[int]] = [[] for _ in range(nranks)]
    for i in order:
        r = min(range(nranks), key=lambda k: (loads[k], k))
        parts[r].append(i)
        loads[r] += float(weights[i])
    return [sorted(p) for p in parts]


def shard_for_rank(weights: Sequence[float], rank: int, world: int) -> List[int]:
    """The systems rank `rank` of `world` steps."""
    return lpt_partition(weights, world)[rank]


def gather_results(local: Dict[int, Any], world: int, group=None) -> Dict[int, Any]:
    """Merges every rank's {system index: result} (torch.distributed, any
    backend); with one process it returns `local`.  A system reported by two
    ranks is an error."""
    if world == 1:
        return dict(local)
    import torch.distributed as dist
    parts: List[Dict[int, Any]] = [None] * world  # type: ignore[list-item]
    dist.all_gather_object(parts, dict(local), group=group)
    merged: Dict[int, Any] = {}
    for p in parts:
        for k, v in p.items():
            if k in merged:
                raise RuntimeError(f"system {k} was stepped by two ranks")
            merged[k] = v
    return merged
