"""Independent replicas on several GPUs (one process per GPU).

The reference scales out by running independent simulations as separate processes, one job
per experiment instance (README.md:148-175, HPC_run_all_exp_distribute.sh:54-75); the hot path
has no cross-swarm exchange, so N GPUs run N replicas, or disjoint instance sets of a batched
sweep, with no data-path collective.  Only the measurement (the slowest rank's time and the
sum of the agent-steps of all ranks) and, on request, the per-instance results are combined.
"""
from __future__ import annotations

import numpy as np
import torch


def shard_instances(sizes, world: int, rank: int) -> np.ndarray:
    """The instances (indices into `sizes`, ascending) that rank `rank` of `world` runs: every
    instance on exactly one rank, balanced by the pair work N_i^2 of its step -- the largest
    instances first, each to the rank with the least work so far (ties to the lower rank).
    Deterministic, so every rank computes the same split without communication."""
    sizes = np.asarray(sizes, np.int64)
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of world {world}")
    load = np.zeros(world, np.int64)
    owner = np.empty(len(sizes), np.int64)
    for k in np.argsort(-sizes, kind="stable"):
        r = int(np.argmin(load))
        owner[k] = r
        load[r] += int(sizes[k]) ** 2
    return np.where(owner == rank)[0]


def gather_instances(local: dict, n_instances: int) -> list:
    """Per-instance results {instance index: value} of every rank, as one list indexed by
    instance on every rank (all_gather_object; the local dict alone without a process
    group)."""
    import torch.distributed as dist
    parts = [local]
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        parts = [None] * dist.get_world_size()
        dist.all_gather_object(parts, local)
    out = [None] * n_instances
    for part in parts:
        for k, v in part.items():
            if out[k] is not None:
                raise RuntimeError(f"instance {k} ran on two ranks")
            out[k] = v
    if any(v is None for v in out):
        raise RuntimeError("an instance ran on no rank")
    return out


def combine(seconds, units: int, device=None):
    """(max over ranks of each entry of `seconds`, sum over ranks of `units`).  Without an
    initialised process group this is the local value."""
    import torch.distributed as dist
    secs = [float(s) for s in seconds]
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return secs, int(units)
    dev = device if device is not None else torch.device("cpu")
    t = torch.tensor(secs, dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    u = torch.tensor([float(units)], dtype=torch.float64, device=dev)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return [float(v) for v in t.cpu()], int(u.item())
