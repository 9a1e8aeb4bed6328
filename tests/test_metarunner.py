"""CPU checks of the batched metarunner front-end (abm_gb300.metarunner) against the
reference's own MetaProtocol (tests/golden/metarunner.json, make_metarunner_golden.py)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN


def _protocol(case, base_env=None, num_batches=1):
    from abm_gb300 import metarunner as mr
    bp = mr.BatchedProtocol(base_env or {}, num_batches=num_batches, experiment_name="exp")
    for c in case["criteria"]:
        if c[0] == "Constant":
            bp.add_criterion(mr.Constant(c[1], c[2]))
        elif isinstance(c[2], list):
            bp.add_criterion(mr.Tunable(c[1], values_override=c[2]))
        else:
            bp.add_criterion(mr.Tunable(c[1], min_v=c[2], max_v=c[3], num_data_points=c[4]))
    for a, b, v in case["pairs"]:
        bp.add_tuned_pair(mr.TunedPairRestrain(a, b, v))
    for a, b, v in case["qpairs"]:
        bp.add_quadratic_tuned_pair(mr.TunedPairRestrain(a, b, v))
    return bp


def test_combinations_match_reference():
    cases = json.load(open(os.path.join(GOLDEN, "metarunner.json")))
    assert len(cases) >= 5
    for case in cases:
        got = _protocol(case).combos()
        want = case["combos"]
        assert len(got) == len(want), case
        for g, w in zip(got, want):
            assert len(g) == len(w)
            for a, b in zip(g, w):
                assert (bool(a) == b) if isinstance(b, bool) else float(a) == b


def test_env_configs_batches_files_and_groups():
    from abm_gb300.params import VFParams
    cases = json.load(open(os.path.join(GOLDEN, "metarunner.json")))
    base = {"ENV_WIDTH": "400", "ENV_HEIGHT": "400", "VF_ALP1": "0.08", "N": "10"}
    bp = _protocol(cases[0], base, num_batches=2)
    envs = bp.env_configs()
    assert len(envs) == 2 * len(cases[0]["combos"])
    assert envs[0]["SAVE_ROOT_DIR"].endswith("exp/batch_0")
    assert envs[-1]["SAVE_ROOT_DIR"].endswith("exp/batch_1")
    assert envs[0]["ENV_WIDTH"] == "400" and float(envs[1]["VF_BET0"]) == 1.0
    names = [n for n, _ in bp.env_files()]
    assert names == sorted(names) and names[0] == "0_b0.env" and "10_b0.env" in names
    # run() writes configuration k into <root>/<its SAVE_ROOT_DIR>/<its .env file stem>
    folders = bp.run_folders("out")
    combos = len(cases[0]["combos"])
    assert len(folders) == len(envs)
    for k, (env, folder) in enumerate(zip(envs, folders)):
        nb, i = divmod(k, combos)
        assert folder == os.path.join("out", env["SAVE_ROOT_DIR"], f"{i}_b{nb}")
    assert sorted(os.path.basename(f) + ".env" for f in folders) == names
    # ALP0 / BET0 / N vary per agent or instance: one batched group
    assert len(bp.groups()) == 1
    insts = bp.instances(seed=3)
    assert all(len(inst["x"]) == 20 for _, inst in insts)   # Constant N = 20
    assert insts[1][1]["bet0"] == 1.0 and "radius" not in insts[1][1]
    # ALP1 differs: one group per value, configurations kept in order within a group
    bp2 = _protocol(cases[2], base)
    groups = bp2.groups()
    alp1 = [VFParams.from_env(e).alp1 for e in bp2.env_configs()]
    assert len(groups) == len(set(alp1))
    for g in groups:
        assert len({alp1[i] for i in g}) == 1 and g == sorted(g)
    # booleans are written as 0 / 1
    bp3 = _protocol(cases[3], base)
    assert {e["AGENT_AGENT_COLLISION"] for e in bp3.env_configs()} == {0, 1}


def test_initial_state_like_vfsimulation():
    from abm_gb300 import metarunner as mr
    env = {"ENV_WIDTH": "600", "ENV_HEIGHT": "480", "N": "50", "RADIUS_AGENT": "10"}
    st = mr.BatchedProtocol.initial_state(env, seed=1)
    r = np.hypot(st["x"] - 300, st["y"] - 240)
    assert len(st["x"]) == 50 and r.max() <= 480 / 2 - 2 * 30 - 10 + 1e-3
    # facing out of the disc (vf_sims.py:217-220)
    ang = np.arctan2(st["y"] - 240, st["x"] - 300) % (2 * np.pi)
    assert np.allclose(ang, st["theta"] % (2 * np.pi), atol=1e-4)
