"""GPU tests of the visual-flocking run recorder (abm_vpf_record, VFSwarm / BatchedSweep
.record_steps) and of the files written from it.

The recorder must hold, column by column, exactly the state after each step and the VPF bitmask
of that step, in eager steps and in replayed graphs alike, stop at its capacity, and the saved
files must carry those values in the reference's layout.
"""
import json
import os

import numpy as np
import pytest

from conftest import gpu_available

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def _swarm(n=60, rv=300, seed=3):
    from abm_gb300.params import VFParams
    from abm_gb300.swarm import VFSwarm
    rng = np.random.default_rng(seed)
    p = VFParams(alp1=0.08, bet1=0.08, width=500.0, height=500.0, rv=rv)
    return VFSwarm(p, rng.uniform(20, 520, n).astype(np.float32),
                   rng.uniform(20, 520, n).astype(np.float32),
                   rng.uniform(0, 2 * np.pi, n).astype(np.float32))


def test_vf_recording_holds_each_step():
    sw = _swarm()
    sw.record_steps(8, vpf=True)
    want = []
    for _ in range(11):          # three steps beyond the capacity are dropped
        sw.step()
        st = sw.state_numpy()
        want.append((st, sw.vpf_bits.cpu().numpy().view(np.uint32).copy()))
    rec = sw.recording()
    assert rec["steps"] == 8
    for t, (st, bits) in enumerate(want[:8]):
        np.testing.assert_array_equal(rec["posx"][:, t], np.trunc(st["x"]).astype(np.int32))
        np.testing.assert_array_equal(rec["posy"][:, t], np.trunc(st["y"]).astype(np.int32))
        np.testing.assert_array_equal(rec["orientation"][:, t], st["theta"])
        np.testing.assert_array_equal(rec["velocity"][:, t], st["v"])
        np.testing.assert_array_equal(rec["vpf_bits"][:, t], bits)


def test_vf_recording_without_vpf_and_files(tmp_path):
    from abm_gb300.recording import read_zarr_array
    sw = _swarm(n=40, rv=256, seed=5)
    sw.record_steps(5)
    for _ in range(5):
        sw.step()
    rec = sw.recording()
    assert "vpf_bits" not in rec and rec["steps"] == 5
    sw.save_reference_run(str(tmp_path / "z"), as_zarr=True, env={"N": "40"})
    x = read_zarr_array(str(tmp_path / "z" / "ag_posx.zarr"))
    # the reference's rows: agent id a in row a - 1, so agent 0 is the last row
    np.testing.assert_array_equal(x, np.roll(rec["posx"], -1, axis=0).astype(np.float64))
    ori = read_zarr_array(str(tmp_path / "z" / "ag_ori.zarr"))
    np.testing.assert_array_equal(ori, np.roll(rec["orientation"], -1, axis=0).astype(np.float64))
    assert np.all(read_zarr_array(str(tmp_path / "z" / "ag_explr.zarr")) == -1.0)
    assert json.load(open(tmp_path / "z" / "env_params.json")) == {"N": "40"}
    sw.save_reference_run(str(tmp_path / "j"))
    d = json.load(open(tmp_path / "j" / "agent_data.json"))
    assert d["3"]["posx"] == [int(v) for v in rec["posx"][3]]
    assert d["3"]["vfield_up"] == []


def test_batched_recording_graph_equals_eager():
    """A sweep recorded through replayed graphs equals the same sweep stepped eagerly; every
    instance's rows hold its own states (several blocks per launch: 2000+ agents x 38 words)."""
    from abm_gb300.batched import BatchedSweep, sweep_instances
    from abm_gb300.params import VFParams
    vp = VFParams(alp1=0.08, bet1=0.08, width=600.0, height=600.0, rv=1200)
    inst = sweep_instances(n_instances=9, n_min=150, n_max=400, alp_grid=(3, 3), seed=21,
                           width=600.0, height=600.0)
    a, b = BatchedSweep(vp, inst), BatchedSweep(vp, inst)
    steps = 2 * 6 + 3
    a.record_steps(steps, vpf=True)
    b.record_steps(steps, vpf=True)
    finals = []
    for _ in range(steps):
        a.step()
    for k in range(len(inst)):
        finals.append(a.instance_state(k))
    b.run(steps, chunk=6)
    for k in range(len(inst)):
        ra, rb = a.instance_recording(k), b.instance_recording(k)
        assert ra["steps"] == rb["steps"] == steps
        for key in ("posx", "posy", "orientation", "velocity", "vpf_bits"):
            np.testing.assert_array_equal(ra[key], rb[key], err_msg=key)
        np.testing.assert_array_equal(ra["orientation"][:, -1], finals[k]["theta"])
        np.testing.assert_array_equal(ra["posx"][:, -1],
                                      np.trunc(finals[k]["x"]).astype(np.int32))


def test_vf_recording_in_library_graph_equals_eager():
    """VFSwarm.run(graph_chunk) with a recorder goes through abm_vpf_flock_run_recorded (step
    and record inside the library's graph): the same records and final state as eager steps,
    for an even and an odd number of steps."""
    import torch
    for steps in (14, 15):
        a, b = _swarm(n=300, rv=600, seed=8), _swarm(n=300, rv=600, seed=8)
        a.record_steps(steps, vpf=True)
        b.record_steps(steps, vpf=True)
        for _ in range(steps):
            a.step()
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())   # b's state was set up there
        b.run(steps, stream=s, graph_chunk=4)
        s.synchronize()
        ra, rb = a.recording(), b.recording()
        assert ra["steps"] == rb["steps"] == steps
        for key in ("posx", "posy", "orientation", "velocity", "vpf_bits"):
            np.testing.assert_array_equal(ra[key], rb[key], err_msg=key)
        for key, val in a.state_numpy().items():
            np.testing.assert_array_equal(val, b.state_numpy()[key], err_msg=key)
