"""Multi-rank replica measurement on CPU: two gloo ranks combine their timings (max) and
agent-step counts (sum) exactly as bench.py does with one process per GPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from abm_gb300.replicas import combine
    secs, units = combine([0.5 + rank, 2.0 - rank], 1000 * (rank + 1))
    out[rank] = (secs, units)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replica_combine():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for r in range(2):
        secs, units = out[r]
        assert secs == [1.5, 2.0]
        assert units == 3000


def test_single_process_is_local():
    from abm_gb300.replicas import combine
    assert combine([1.0, 2.0], 7) == ([1.0, 2.0], 7)
