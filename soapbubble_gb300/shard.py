"""Sharding of independent bubbles across ranks (one process per GPU).

The ensemble and the serving stream are made of independent bubbles: no
bubble reads another's state, so a rank steps its own bubbles and no field
data moves between ranks.  The only traffic between ranks is host-side
bookkeeping around the timed region: a barrier before and after it and the
maximum of the elapsed times (torch.distributed on the host; gloo suffices,
nothing on the data path needs NCCL).  A single bubble does not shard (its
implicit solve couples every cell every iteration): ranks then run
independent replicas.

Partitions are deterministic functions of the workload, the world size and
the rank, so every rank computes the same assignment without exchanging it.
"""
from __future__ import annotations

import os
import time
from typing import Callable, List, Optional, Sequence, Tuple


def partition(weights: Sequence[float], world: int) -> List[List[int]]:
    """Longest-processing-time partition: items by decreasing weight (ties by
    index) go to the least loaded rank (ties to the lowest rank).  Every
    rank's load is within the largest item of the average.  Returns the item
    indices of every rank in increasing order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    load = [0.0] * world
    parts: List[List[int]] = [[] for _ in range(world)]
    for k in sorted(range(len(weights)), key=lambda i: (-float(weights[i]), i)):
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(k)
        load[r] += float(weights[k])
    return [sorted(p) for p in parts]


def member_weight(nTheta: int, steps: int = 1) -> float:
    """Work of a bubble: cells x steps (nPhi = 2 nTheta)."""
    return 2.0 * nTheta * nTheta * steps


def shard_members(members, world: int, rank: int) -> list:
    """The ensemble members (objects with .nTheta) rank `rank` steps."""
    idx = partition([member_weight(m.nTheta) for m in members], world)[rank]
    return [members[k] for k in idx]


def shard_requests(requests, world: int, rank: int) -> list:
    """The serving requests (objects with .nTheta, .steps, .arrival) rank
    `rank` serves, in arrival order: the stream is known when it is
    generated, so it is split by work (cells x steps) up front."""
    idx = partition([member_weight(r.nTheta, r.steps) for r in requests], world)[rank]
    return sorted((requests[k] for k in idx), key=lambda r: (r.arrival, r.rid))


class Ranks:
    """World size, rank and host-side collectives of this process
    (RANK / WORLD_SIZE / LOCAL_RANK / MASTER_* from the environment, as
    torchrun sets them; one process without them)."""

    def __init__(self, backend: str = "gloo"):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        if self.world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group(backend)
            self.dist = dist

    def barrier(self) -> None:
        if self.dist is not None:
            self.dist.barrier()

    def _reduce(self, x: float, op: str) -> float:
        if self.dist is None:
            return float(x)
        import torch
        t = torch.tensor([float(x)], dtype=torch.float64)
        self.dist.all_reduce(t, op=getattr(self.dist.ReduceOp, op))
        return float(t.item())

    def max(self, x: float) -> float:
        return self._reduce(x, "MAX")

    def sum(self, x: float) -> float:
        return self._reduce(x, "SUM")


def timed_shard(ranks: Ranks, work: Callable[[], Tuple[float, Optional[float]]]) -> dict:
    """Runs this rank's share between two barriers.  work() returns (units
    processed by this rank, its own elapsed seconds or None to use the
    host clock between the barriers).  The job's throughput is the units
    of all ranks over the slowest rank's time."""
    ranks.barrier()
    t0 = time.perf_counter()
    units, own = work()
    ranks.barrier()
    host = time.perf_counter() - t0
    el = own if own is not None else host
    total = ranks.sum(units)
    el_max = ranks.max(el)
    return {"units": total, "seconds_max": el_max, "value": total / el_max if el_max > 0 else 0.0,
            "units_rank": units, "seconds_rank": el, "world": ranks.world}


def run_ensemble_shard(members, steps: int, dt: float, ranks: Ranks, device: Optional[int] = None,
                       autotune: bool = True) -> dict:
    """The batched ensemble on this rank's members (one set per rank, its
    own GPU); throughput over all ranks."""
    from . import ensemble
    mine = shard_members(members, ranks.world, ranks.rank)
    if not mine:  # more ranks than members
        out = timed_shard(ranks, lambda: (0.0, 0.0))
        out["members_rank"] = 0
        return out
    dev = ranks.local if device is None else device
    fields = ensemble.member_fields(mine)
    bubbles = ensemble.make_bubbles(mine, fields, dt, solver_mode=0, device=dev)

    def work():
        r = ensemble.run_batched(bubbles, steps, dt, autotune=autotune)
        return ensemble.cells(mine) * steps, r["ms_per_step"] * steps / 1e3

    try:
        out = timed_shard(ranks, work)
    finally:
        for g in bubbles:
            g.close()
    out["members_rank"] = len(mine)
    return out
