"""Independent instances across ranks: one process per GPU, no data exchange.

The march of one instance does not shard without an all-to-all transpose of the
whole field twice per spectral stage (the t-column passes are independent per
(x, y) column, the plane passes per frequency plane). Independent instances —
transducer configurations, steering foci, parameter sweeps — are the unit that
shards: each rank marches its own instances and only host-side summaries and
timings cross ranks.

The reference has no multi-device path (its march is a single JAX program,
angular_spectrum_solver.py:1408-1550); this module is the host logic around
replicas of `angular_spectrum_solve`.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any, Callable, Dict, List, Sequence


@dataclass(frozen=True)
class Instance:
    """One independent march: a grid, a step count and a free-form payload."""
    index: int
    shape: tuple          # (nX, nY, nT)
    steps: int
    payload: Any = None

    @property
    def voxel_steps(self) -> int:
        nx, ny, nt = self.shape
        return nx * ny * nt * self.steps


def partition(costs: Sequence[float], world_size: int) -> List[List[int]]:
    """Longest-processing-time-first assignment of instances to ranks.

    Returns, for each rank, the indices of its instances in ascending order.
    Deterministic: ties in cost go to the lower index, ties in load to the
    lower rank, so every rank computes the same partition without talking.
    """
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world_size
    out: List[List[int]] = [[] for _ in range(world_size)]
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += float(costs[i])
    return [sorted(o) for o in out]


def rank_env():
    """(rank, world_size, local_rank) from the torchrun environment."""
    import os
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def max_over_ranks(value: float, device=None) -> float:
    """The largest `value` over all ranks (the job's wall time is the slowest
    rank's). Without an initialised process group, `value` itself."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64,
                     device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_instances(instances: Sequence[Instance], solve: Callable[[Instance], Any],
                  summarize: Callable[[Instance, Any], Dict] = None) -> Dict[int, Dict]:
    """March this rank's share of `instances` and gather summaries on rank 0.

    `solve(inst)` runs one instance (normally a wrapper around
    `angular_spectrum_solve`); `summarize(inst, result)` reduces its output to
    a small picklable dict (focal pnp/ppp/pI, timings) — full fields stay on
    the rank that made them. Returns {index: summary} for every instance on
    rank 0, and for this rank's instances elsewhere.
    """
    import torch.distributed as dist
    dist_on = dist.is_available() and dist.is_initialized()
    rank = dist.get_rank() if dist_on else 0
    world = dist.get_world_size() if dist_on else 1
    mine = partition([i.voxel_steps for i in instances], world)[rank]
    local = {}
    for k in mine:
        inst = instances[k]
        res = solve(inst)
        local[inst.index] = summarize(inst, res) if summarize else {"result": res}
        local[inst.index]["rank"] = rank
    if not dist_on:
        return local
    gathered = [None] * world if rank == 0 else None
    dist.gather_object(local, gathered, dst=0)
    if rank != 0:
        return local
    out = {}
    for part in gathered:
        out.update(part)
    return out
