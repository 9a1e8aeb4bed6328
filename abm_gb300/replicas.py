"""Independent replicas on several GPUs (one process per GPU).

The reference scales out by running independent simulations as separate processes
(README.md:148-175, HPC_run_all_exp_distribute.sh); the hot path has no cross-swarm exchange,
so N GPUs run N replicas (or disjoint instance sets of a batched sweep) with no data-path
collective.  Only the measurement is combined: the slowest rank's time and the sum of the
agent-steps of all ranks.
"""
from __future__ import annotations

import torch


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
