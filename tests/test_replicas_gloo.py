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


def test_shards_are_disjoint_cover_and_balanced():
    import numpy as np
    from abm_gb300.replicas import shard_instances
    sizes = np.random.default_rng(3).integers(10, 501, 512)
    for world in (1, 2, 3, 4, 8):
        shards = [shard_instances(sizes, world, r) for r in range(world)]
        allk = np.concatenate(shards)
        assert np.array_equal(np.sort(allk), np.arange(len(sizes)))
        loads = np.array([np.sum(sizes[s].astype(np.int64) ** 2) for s in shards])
        # greedy by decreasing size: no rank exceeds the mean by more than one instance
        assert loads.max() <= loads.sum() / world + sizes.max() ** 2


def _shard_worker(rank, world, port, out):
    """Each rank steps only its shard of a small sweep with the oracle (FP64 C restatement of
    the reference step) and the per-instance results are gathered on every rank."""
    import numpy as np
    import torch.distributed as dist
    import oracle
    from abm_gb300.replicas import shard_instances, gather_instances
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    insts, p = _sweep()
    mine = shard_instances([len(d["x"]) for d in insts], world, rank)
    local = {int(k): oracle.vf_step(insts[k], dict(p, alp0=insts[k]["alp0"]),
                                    want_vpf=False, want_terms=False)["theta"]
             for k in mine}
    res = gather_instances(local, len(insts))
    out[rank] = ([int(k) for k in mine], [r.tolist() for r in res])
    dist.barrier()
    dist.destroy_process_group()


def _sweep():
    import numpy as np
    rng = np.random.default_rng(12)
    insts = []
    for k in range(9):
        n = int(rng.integers(2, 40))
        insts.append({"x": rng.uniform(20, 420, n), "y": rng.uniform(20, 420, n),
                      "theta": rng.uniform(0, 2 * np.pi, n), "v": rng.uniform(0, 1, n),
                      "alp0": 0.5 + 0.1 * k})
    p = dict(gam=0.1, v0=1.0, alp0=1.0, alp1=0.08, alp2=0.0, bet0=1.0, bet1=0.08, bet2=0.0,
             boundary=0, limit_movement=0, max_vel=3.0, max_th=0.1, width=400.0,
             height=400.0, window_pad=30.0, fov0=-3.141592653589793,
             fov1=3.141592653589793, rv=240, radius=10.0, dt=1.0)
    return insts, p


def test_two_rank_sharded_sweep_equals_one_rank():
    """Two gloo ranks run disjoint halves of a sweep; the gathered per-instance results equal
    the single-process results of every instance."""
    import numpy as np
    import oracle
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
        assert p.exitcode == 0
    insts, p = _sweep()
    want = [oracle.vf_step(d, dict(p, alp0=d["alp0"]), want_vpf=False,
                           want_terms=False)["theta"] for d in insts]
    mine0, res0 = out[0]
    mine1, res1 = out[1]
    assert sorted(mine0 + mine1) == list(range(len(insts))) and not set(mine0) & set(mine1)
    assert res0 == res1
    for k, w in enumerate(want):
        assert np.array_equal(np.array(res0[k]), w), k
