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
