"""GPU test of the batched metarunner front-end: every configuration of a protocol run as
batched launches ends in the same state as that configuration run alone."""
import numpy as np
import pytest

from conftest import gpu_available

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def test_protocol_runs_match_single_runs():
    from abm_gb300 import metarunner as mr
    from abm_gb300.params import VFParams
    from abm_gb300.swarm import VFSwarm
    base = {"ENV_WIDTH": "400", "ENV_HEIGHT": "400", "VISUAL_FIELD_RESOLUTION": "600",
            "RADIUS_AGENT": "10"}
    bp = mr.BatchedProtocol(base, num_batches=2)
    bp.add_criterion(mr.Tunable("VF_ALP0", values_override=[0.5, 1.5]))
    bp.add_criterion(mr.Tunable("VF_ALP1", values_override=[0.05, 0.1]))
    bp.add_criterion(mr.Tunable("N", values_override=[12, 30]))
    assert len(bp.groups()) == 2
    steps = 130
    results = bp.run(steps, seed=7, chunk=100)
    envs = bp.env_configs()
    assert len(results) == len(envs) == 16
    for idx, env in enumerate(envs):
        p = VFParams.from_env(env)
        st = mr.BatchedProtocol.initial_state(env, 7 + idx)
        n = len(st["x"])
        sw = VFSwarm(p, st["x"], st["y"], st["theta"], st["v"], alp0=np.full(n, p.alp0),
                     bet0=np.full(n, p.bet0))
        for _ in range(steps):
            sw.step()
        want = sw.state_numpy()
        for k in want:
            assert np.array_equal(results[idx][k], want[k]), (idx, k)


def test_protocol_saves_runs_like_single_runs(tmp_path):
    """run(save_root=...) writes each configuration's data (JSON or zarr by its
    USE_ZARR_FORMAT, and env_params.json) exactly as a single recorded run of it writes them."""
    import json
    import os

    from abm_gb300 import metarunner as mr
    from abm_gb300.params import VFParams
    from abm_gb300.recording import read_zarr_array
    from abm_gb300.swarm import VFSwarm
    base = {"ENV_WIDTH": "400", "ENV_HEIGHT": "400", "VISUAL_FIELD_RESOLUTION": "600",
            "RADIUS_AGENT": "10", "N": "15", "USE_ZARR_FORMAT": "0"}
    bp = mr.BatchedProtocol(base, num_batches=1, experiment_name="rec")
    bp.add_criterion(mr.Tunable("VF_ALP0", values_override=[0.5, 1.5]))
    bp.add_criterion(mr.Tunable("USE_ZARR_FORMAT", values_override=[0, 1]))
    steps = 14
    bp.run(steps, seed=3, chunk=4, save_root=str(tmp_path / "out"))
    folders = bp.run_folders(str(tmp_path / "out"))
    assert folders[0].endswith(os.path.join("rec", "batch_0", "0_b0"))
    for idx, (env, folder) in enumerate(zip(bp.env_configs(), folders)):
        p = VFParams.from_env(env)
        st = mr.BatchedProtocol.initial_state(env, 3 + idx)
        n = len(st["x"])
        sw = VFSwarm(p, st["x"], st["y"], st["theta"], st["v"], alp0=np.full(n, p.alp0),
                     bet0=np.full(n, p.bet0))
        sw.record_steps(steps, vpf=True)
        for _ in range(steps):
            sw.step()
        zarr = bool(int(env["USE_ZARR_FORMAT"]))
        single = str(tmp_path / f"single{idx}")
        sw.save_reference_run(single, as_zarr=zarr, env={k: f"{v}" for k, v in env.items()})
        assert json.load(open(os.path.join(folder, "env_params.json"))) == \
            json.load(open(os.path.join(single, "env_params.json")))
        if zarr:
            names = sorted(f for f in os.listdir(folder) if f.endswith(".zarr"))
            assert names == sorted(f for f in os.listdir(single) if f.endswith(".zarr"))
            assert "ag_posx.zarr" in names
            for name in names:
                assert np.array_equal(read_zarr_array(os.path.join(folder, name)),
                                      read_zarr_array(os.path.join(single, name))), name
        else:
            for name in ("agent_data.json", "resource_data.json"):
                assert open(os.path.join(folder, name)).read() == \
                    open(os.path.join(single, name)).read(), name
