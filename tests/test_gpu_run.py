"""GPU tests of the multi-step entry points abm_vpf_flock_run / abm_vpf_flock_batched_run:
one library call that replays a CUDA graph of graph_chunk steps gives, bit for bit, the state of
the same number of single-step calls, for every parity of the step count and chunk size."""
import ctypes

import numpy as np
import pytest
import torch

from conftest import gpu_available

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def _swarm(seed=5, n=300):
    from abm_gb300.params import VFParams
    from abm_gb300.swarm import VFSwarm
    rng = np.random.default_rng(seed)
    W = 600.0
    x = rng.uniform(20, 20 + W, n).astype(np.float32)
    y = rng.uniform(20, 20 + W, n).astype(np.float32)
    th = rng.uniform(0, 2 * np.pi, n).astype(np.float32)
    p = VFParams(alp1=0.08, bet1=0.08, width=W, height=W, rv=1200, radius=5.0)
    return lambda: VFSwarm(p, x, y, th, device="cuda")


@pytest.mark.parametrize("steps,chunk", [(1, 10), (7, 4), (10, 4), (23, 6), (12, 0), (9, 2)])
def test_flock_run_matches_single_steps(steps, chunk):
    make = _swarm()
    a, b = make(), make()
    for _ in range(steps):
        a.step()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    b.run(steps, stream=side, graph_chunk=chunk)
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    sa, sb = a.state_numpy(), b.state_numpy()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), (steps, chunk, k)


@pytest.mark.parametrize("steps,chunk", [(8, 4), (11, 4)])
def test_batched_run_matches_single_steps(steps, chunk):
    from abm_gb300 import _lib
    from abm_gb300.batched import BatchedSweep, sweep_instances
    from abm_gb300.params import VFParams
    vp = VFParams(gam=0.1, v0=1.0, alp1=0.08, bet1=0.08, width=500.0, height=500.0, rv=400,
                  radius=10.0)
    inst = sweep_instances(n_instances=24, n_min=5, n_max=60, width=500.0, height=500.0,
                           seed=8)
    a, b = BatchedSweep(vp, inst), BatchedSweep(vp, inst)
    for _ in range(steps):
        a.step()
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    s0, s1 = b._state(b._bufs[b._cur]), b._state(b._bufs[1 - b._cur])
    st = b.lib.abm_vpf_flock_batched_run(
        ctypes.byref(s0), ctypes.byref(s1), b.n, _lib.i32ptr(b.seg_begin), _lib.i32ptr(b.seg_end),
        _lib.i32ptr(b.order), ctypes.byref(b._cparams), ctypes.byref(b._ov), steps, chunk,
        _lib.u64ptr(b.diag), ctypes.c_void_p(side.cuda_stream))
    assert st >= 0, _lib.load().abm_last_error_string()
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    fin = b._bufs[b._cur if steps % 2 == 0 else 1 - b._cur]
    cur_a = a._bufs[a._cur]
    for k in ("x", "y", "theta", "v"):
        assert np.array_equal(cur_a[k].cpu().numpy(), fin[k].cpu().numpy()), (steps, chunk, k)


def test_run_rejects_bad_arguments():
    from abm_gb300 import _lib
    make = _swarm()
    s = make()
    st = s.lib.abm_vpf_flock_run(None, None, s.n, ctypes.byref(s._cparams), None, 4, 2, None,
                                 None)
    assert st == _lib.ABM_ERR_INVALID_ARG


@pytest.mark.parametrize("collide,steps,chunk", [(False, 250, 100), (True, 130, 40),
                                                 (False, 7, 100)])
def test_forage_run_matches_single_steps(collide, steps, chunk):
    """abm_forage_run (library graph of graph_chunk steps) = single abm_forage_step calls,
    recording included."""
    from abm_gb300.foraging import ForageParams, ForagingSim
    prm = ForageParams(seed=12, min_resc_units=20, max_resc_units=60, collide_agents=collide,
                       width=400.0, height=400.0, rv=400)
    a = ForagingSim(prm, n_agents=60, n_patches=3, init_seed=4, record_steps=steps)
    b = ForagingSim(prm, n_agents=60, n_patches=3, init_seed=4, record_steps=steps)
    for _ in range(steps):
        a.step()
    b.run_in_library(steps, graph_chunk=chunk)
    torch.cuda.synchronize()
    sa, sb = a.agents_numpy(), b.agents_numpy()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    pa, pb = a.patches_numpy(), b.patches_numpy()
    for k in pa:
        assert np.array_equal(pa[k], pb[k]), k
    ra, rb = a.recording(), b.recording()
    for k in ra:
        assert np.array_equal(np.asarray(ra[k]), np.asarray(rb[k])), k
