"""Placement of independent scenes on the ranks of a multi-GPU job.

Scenes never exchange data, so a batch or a request stream shards by whole
scenes with no collective on the data path; the only cross-rank traffic is
the timing and metric reduction at the end.  A single scene is not split:
runs of one scene on N GPUs are N replicas.
"""
from __future__ import annotations


def request_cost(r: dict) -> float:
    """Work of a request in particle-steps (at least one step's worth)."""
    return float(r["particles"]) * max(int(r.get("steps", 0)), 1)


def shard_requests(reqs: list, world: int, rank: int) -> list:
    """Longest-processing-time placement: requests sorted by decreasing cost
    (ties by position) go to the least-loaded rank (ties to the lowest rank).
    Every rank computes the same placement from the same list and keeps its
    own share, in the original order.  The largest share is within one
    request of 4/3 of the optimum (Graham's bound)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world/rank")
    order = sorted(range(len(reqs)), key=lambda i: (-request_cost(reqs[i]), i))
    load = [0.0] * world
    owner = [0] * len(reqs)
    for i in order:
        k = min(range(world), key=lambda r: (load[r], r))
        owner[i] = k
        load[k] += request_cost(reqs[i])
    return [reqs[i] for i in range(len(reqs)) if owner[i] == rank]


def shard_loads(reqs: list, world: int) -> list:
    return [sum(request_cost(r) for r in shard_requests(reqs, world, k)) for k in range(world)]
