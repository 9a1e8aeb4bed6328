"""GPU tests of the launch-configuration autotuner (abm_vpf_autotune / abm_gb300.autotune)."""
import ctypes

import numpy as np
import pytest

from conftest import gpu_available
from _gpu_helpers import seeded_swarm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


@pytest.fixture
def restore_config():
    from abm_gb300 import _lib
    lib = _lib.load()
    yield
    lib.abm_vpf_set_step_mode(0, 1)
    lib.abm_vpf_set_step_config(8, 8192)
    lib.abm_vpf_set_step_split(0)


def _current(lib):
    m, w, wb, t, c = (ctypes.c_int32() for _ in range(5))
    lib.abm_vpf_get_step_mode(ctypes.byref(m), ctypes.byref(w))
    lib.abm_vpf_get_step_config(ctypes.byref(wb), ctypes.byref(t))
    lib.abm_vpf_get_step_split(ctypes.byref(c))
    return {"mode": m.value, "warps_per_agent": w.value, "warps_per_block": wb.value,
            "tile": t.value, "chunks": c.value}


def test_autotune_single_swarm(restore_config):
    """33 candidates; the chosen one is the fastest measured and is applied; the step under
    it is bit-identical to the step under the default configuration."""
    from abm_gb300 import _lib, autotune
    from abm_gb300.params import VFParams
    from abm_gb300.swarm import VFSwarm
    lib = _lib.load()
    st = seeded_swarm(21, 1500, 2500.0, 2500.0, R=5.0)
    vp = VFParams(width=2500.0, height=2500.0, rv=2000, radius=5.0)
    ref = VFSwarm(vp, st["x"], st["y"], st["theta"], st["v"])
    ref.step(want_vpf=True, want_terms=True)
    want = (ref.vpf_numpy(), ref.terms.cpu().numpy(), ref.state_numpy())

    s = VFSwarm(vp, st["x"], st["y"], st["theta"], st["v"])
    res = autotune.tune(s, reps=2)
    tried = res["tried"]
    assert len(tried) == 33   # 6 group-form + 15 L1-form + 12 tiled-form candidates
    ran = [t for t in tried if t["ms_per_step"] > 0]
    assert ran, tried
    best = res["best"]
    assert best["ms_per_step"] == min(t["ms_per_step"] for t in ran)
    cur = _current(lib)
    for k in ("mode", "warps_per_agent", "chunks"):
        assert cur[k] == best[k]
    if best["mode"] == 2:
        assert cur["warps_per_block"] == best["warps_per_block"] and cur["tile"] == best["tile"]
    s.step(want_vpf=True, want_terms=True)
    got = (s.vpf_numpy(), s.terms.cpu().numpy(), s.state_numpy())
    assert np.array_equal(got[0], want[0])
    assert np.array_equal(got[1], want[1])
    for k in want[2]:
        assert np.array_equal(got[2][k], want[2][k])


def test_autotune_batched_sweep(restore_config):
    """A batched sweep has the three warps-per-agent candidates of the segmented L1 form; its
    state is not changed by tuning and the tuned step matches per-instance steps."""
    from abm_gb300 import _lib, autotune
    from abm_gb300.batched import BatchedSweep, sweep_instances
    from abm_gb300.params import VFParams
    from abm_gb300.swarm import VFSwarm
    lib = _lib.load()
    inst = sweep_instances(n_instances=9, n_min=10, n_max=200, alp_grid=(3, 3), seed=5,
                           width=600.0, height=600.0)
    vp = VFParams(alp1=0.08, bet1=0.08, width=600.0, height=600.0, rv=1200)
    b = BatchedSweep(vp, inst)
    before = {k: t.clone() for k, t in b._bufs[b._cur].items()}
    res = autotune.tune(b, reps=2)
    assert len(res["tried"]) == 4   # the group form, and the L1 form with 1, 2, 4 warps
    assert [t["mode"] for t in res["tried"]] == [3, 1, 1, 1]
    assert all(t["chunks"] == 1 for t in res["tried"])
    for k, t in before.items():
        assert bool((b._bufs[b._cur][k] == t).all())
    assert _current(lib)["warps_per_agent"] == res["best"]["warps_per_agent"]
    b.step()
    for k in range(len(inst)):
        n = len(inst[k]["x"])
        s = VFSwarm(vp, inst[k]["x"], inst[k]["y"], inst[k]["theta"], inst[k]["v"],
                    alp0=np.full(n, inst[k]["alp0"]), bet0=np.full(n, inst[k]["bet0"]))
        s.step()
        got, want = b.instance_state(k), s.state_numpy()
        for key in want:
            assert np.array_equal(got[key], want[key]), (k, key)
