"""GPU tests of the foraging step (abm_forage_step / abm_gb300.foraging): against fixtures of
the reference's own step, against the oracle step by step (same random stream), graph replay
and determinism."""
import numpy as np
import pytest
import torch

import oracle
from conftest import gpu_available, load_cases
from test_forage_oracle import AGENT_INT, _ulps32

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def _check(a, p, soc, want_a, want_p, want_soc, tag):
    assert np.array_equal(soc, want_soc), tag
    for k in AGENT_INT + ("draws",):
        if k in want_a:
            assert np.array_equal(np.asarray(a[k]).astype(np.int64),
                                  np.asarray(want_a[k]).astype(np.int64)), (tag, k)
    for k in ("w", "u", "collected", "collected_before"):
        np.testing.assert_allclose(a[k], want_a[k], rtol=0, atol=1e-12, err_msg=f"{tag} {k}")
    for k in ("x", "y", "theta", "v"):
        assert np.max(_ulps32(a[k], want_a[k])) <= 2.0, (tag, k)
    for k in want_p:
        if k in ("x", "y", "radius", "units", "left", "quality"):
            assert np.array_equal(p[k], want_p[k]), (tag, k)
        else:
            assert np.array_equal(np.asarray(p[k]).astype(np.int64),
                                  np.asarray(want_p[k]).astype(np.int64)), (tag, k)


@pytest.mark.parametrize("fixture", ["forage", "collision"])
def test_forage_step_matches_reference_fixtures(fixture):
    """One step from each fixture state against the reference's own step (the collision
    fixtures run its agent-agent block first)."""
    from abm_gb300.foraging import ForageParams, ForagingSim
    for ci, c in enumerate(load_cases(fixture)):
        prm = ForageParams.from_arrays(c["fp"], c["ip"], 0)
        ag = {k[3:]: v for k, v in c.items() if k.startswith("in_")}
        pt = {k[4:]: v for k, v in c.items() if k.startswith("pin_")}
        sim = ForagingSim(prm, agents=ag, patches=pt)
        sim.step(uniforms=torch.as_tensor(c["uniforms"], dtype=torch.float64, device="cuda"))
        want_a = {k[4:]: v for k, v in c.items() if k.startswith("out_")}
        want_p = {k[5:]: v for k, v in c.items() if k.startswith("pout_")}
        rv = int(c["ip"][7])
        _check(sim.agents_numpy(), sim.patches_numpy(), sim.soc_numpy(), want_a, want_p,
               np.unpackbits(c["soc"], axis=1)[:, :rv], f"case {ci}")


@pytest.mark.parametrize("seed,teleport,pooling", [(3, True, 0), (4, False, 0), (5, True, 2)])
def test_forage_step_matches_oracle_every_step(seed, teleport, pooling):
    """120 steps of a 40-agent arena with small patches (depletion and regeneration happen),
    each compared with the oracle step from the same state (identical Philox draws)."""
    from abm_gb300.foraging import ForageParams, ForagingSim
    prm = ForageParams(seed=seed, width=400.0, height=400.0, rv=400, min_resc_units=5,
                       max_resc_units=30, min_resc_quality=0.5, max_resc_quality=1.5,
                       teleport_exploit=teleport, pooling_time=pooling, vision_range=300.0)
    sim = ForagingSim(prm, n_agents=40, n_patches=4, init_seed=seed)
    fp, ip, s = prm.oracle_arrays()
    regenerated = 0
    for t in range(120):
        a0, p0 = sim.agents_numpy(), sim.patches_numpy()
        sim.step()
        a1, p1, soc, failed = oracle.forage_step(a0, p0, fp, ip, s)
        _check(sim.agents_numpy(), sim.patches_numpy(), sim.soc_numpy(), a1, p1,
               soc.astype(np.uint8), f"step {t}")
        regenerated += int(np.sum(p1["draws"] != p0["draws"]))
    if pooling == 0:
        assert regenerated >= 1
    else:
        # sims.py:821-823 notifies an agent only when it relocates or pools with pool_success
        # set, and only a notification sets pool_success: agents starting at 0 never exploit
        assert sim.collected().sum() == 0


@pytest.mark.parametrize("seed,ghost,teleport,rv", [(21, True, True, 400), (22, False, True, 121),
                                                    (23, True, False, 1200),
                                                    (24, False, False, 120)])
def test_collision_step_matches_oracle_every_step(seed, ghost, teleport, rv):
    """A crowded arena with agent-agent collisions (60 agents on 250 x 250): 80 steps, each
    compared with the oracle step from the same state."""
    from abm_gb300.foraging import ForageParams, ForagingSim
    prm = ForageParams(seed=seed, width=250.0, height=250.0, rv=rv, min_resc_units=5,
                       max_resc_units=30, teleport_exploit=teleport, vision_range=200.0,
                       collide_agents=True, ghost_mode=ghost)
    sim = ForagingSim(prm, n_agents=60, n_patches=3, init_seed=seed)
    fp, ip, s = prm.oracle_arrays()
    collided = 0
    for t in range(80):
        a0, p0 = sim.agents_numpy(), sim.patches_numpy()
        sim.step()
        a1, p1, soc, failed = oracle.forage_step(a0, p0, fp, ip, s)
        _check(sim.agents_numpy(), sim.patches_numpy(), sim.soc_numpy(), a1, p1,
               soc.astype(np.uint8), f"step {t}")
        collided += int(np.sum(a1["override_mode"] == 4))
    assert collided >= 40


@pytest.mark.parametrize("collide", [False, True])
def test_forage_graph_replay_and_determinism(collide):
    """A 100-step graph replay gives the eager steps' state; the same seed gives the same run."""
    from abm_gb300.foraging import ForageParams, ForagingSim
    prm = ForageParams(seed=9, min_resc_units=20, max_resc_units=60, collide_agents=collide)
    a = ForagingSim(prm, n_agents=100, n_patches=3, init_seed=2)
    b = ForagingSim(prm, n_agents=100, n_patches=3, init_seed=2)
    for _ in range(200):
        a.step()
    b.run(200, chunk=100)
    torch.cuda.synchronize()
    sa, sb = a.agents_numpy(), b.agents_numpy()
    for k in sa:
        assert np.array_equal(sa[k], sb[k]), k
    pa, pb = a.patches_numpy(), b.patches_numpy()
    for k in pa:
        assert np.array_equal(pa[k], pb[k]), k
    assert a.collected().sum() > 0


def test_forage_efficiency_ensemble_matches_reference():
    """Long runs: the mean foraging efficiency (data_loader.py:1333-1346) of GPU runs (snapshot
    updates, Philox draws) agrees with whole runs of the reference's own sequential loop
    (tests/golden/make_forage_ensemble.py) from the same initial placements, within four
    combined standard errors of the run means."""
    import os
    from conftest import GOLDEN
    from abm_gb300.foraging import ForageParams, ForagingSim, efficiency, initial_state
    z = np.load(os.path.join(GOLDEN, "forage_ensemble.npz"))
    ref = z["eff"].mean(axis=1)                    # per run
    T, T0 = int(z["T"]), int(z["T0"])
    runs = []
    for seed in z["seeds"]:
        for rep in range(4):
            prm = ForageParams.from_arrays(z["fp"], z["ip"], seed=int(seed) * 16 + rep)
            ag, pt = initial_state(prm, int(z["n_agents"]), int(z["n_patches"]), seed=int(seed))
            sim = ForagingSim(prm, agents=ag, patches=pt)
            sim.run(T0, chunk=100)
            c0 = sim.collected()
            sim.run(T - T0, chunk=100)
            runs.append(efficiency(c0, sim.collected(), T - T0).mean())
    gpu = np.array(runs)
    se = np.sqrt(gpu.var(ddof=1) / len(gpu) + ref.var(ddof=1) / len(ref))
    assert abs(gpu.mean() - ref.mean()) <= 4 * se, (gpu.mean(), ref.mean(), se)
    assert gpu.mean() > 0.01


def test_forage_recording_matches_states_and_graph_replay():
    """The device recorder holds, for every step, the state after that step (modes in the
    reference's codes, positions truncated like int()) and its social field; a graph-replayed
    recording equals the eager one; the saved files are the reference's JSON layout."""
    import json
    import tempfile
    from abm_gb300.foraging import ForageParams, ForagingSim
    prm = ForageParams(seed=21, width=500.0, height=500.0, rv=300, min_resc_units=20,
                       max_resc_units=60)
    a = ForagingSim(prm, n_agents=40, n_patches=3, init_seed=4, record_steps=300)
    b = ForagingSim(prm, n_agents=40, n_patches=3, init_seed=4, record_steps=300)
    code = {0: 0, 2: 1, 1: 2, 4: 3}
    states, socs = [], []
    for _ in range(200):
        a.step()
        states.append(a.agents_numpy())
        socs.append(a.soc_bits.cpu().numpy().view(np.uint32))
    b.run(200, chunk=100)
    ra, rb = a.recording(), b.recording()
    assert ra["steps"] == rb["steps"] == 200
    for k in ("posx", "posy", "orientation", "velocity", "w", "u", "ipriv", "collected",
              "mode", "patch_id", "res_left", "res_id", "soc_bits"):
        assert np.array_equal(ra[k], rb[k]), k
    for t, st in enumerate(states):
        assert np.array_equal(ra["posx"][:, t], st["x"].astype(np.int32))
        assert np.array_equal(ra["orientation"][:, t], st["theta"])
        assert np.array_equal(ra["collected"][:, t], st["collected"])
        assert np.array_equal(ra["mode"][:, t], [code[int(m)] for m in st["mode"]])
        assert np.array_equal(ra["soc_bits"][:, t], socs[t])
    with tempfile.TemporaryDirectory() as d:
        a.save_reference_json(d, env={"N": "40", "VISUAL_FIELD_RESOLUTION": "300"})
        ag = json.load(open(f"{d}/agent_data.json"))
        rs = json.load(open(f"{d}/resource_data.json"))
        env = json.load(open(f"{d}/env_params.json"))
    assert len(ag) == 40 and len(ag["0"]["posx"]) == 200 and ag["7"]["agent_name"] == "agent-07"
    assert all(len(v["vfield_up"]) == len(v["vfield_down"]) == 200 for v in ag.values())
    assert len(rs) >= 3 and env["N"] == "40"
    from abm_gb300.recording import read_zarr_array
    with tempfile.TemporaryDirectory() as d:
        names = a.save_reference_zarr(d)
        assert "ag_posx" in names and "res_left" in names and "ag_vf" not in names
        x = read_zarr_array(f"{d}/ag_posx.zarr")
        coll = read_zarr_array(f"{d}/ag_collr.zarr")
        left = read_zarr_array(f"{d}/res_left.zarr")
    # agent id a in row a - 1 (agent 0 last), patch id p in row p - 1
    assert np.array_equal(x, np.roll(ra["posx"], -1, axis=0).astype(np.float64))
    assert np.array_equal(coll, np.roll(ra["collected"], -1, axis=0))
    assert left.shape == (len(rs), 200)
    for rid, r in rs.items():
        assert np.array_equal(left[int(rid) - 1], r["resc_left"])


@pytest.mark.parametrize("rv", [1200, 1201, 400])
def test_collision_exact_paths_match_oracle(rv):
    """Mirror-symmetric neighbours (equal pixel counts in the two halves: the half comparison
    is a tie that numpy's rounding decides) and neighbours exactly ahead or behind (bearings on
    the field's limits): the kernel takes its exact routes (pairwise-sum replay, FP64
    bearings; counted in the diagnostics) and still equals the oracle."""
    from abm_gb300.foraging import ForageParams, ForagingSim, initial_state
    prm = ForageParams(width=1000.0, height=1000.0, rv=rv, fov=1.0, teleport_exploit=False,
                       collide_agents=True, ghost_mode=True, vision_range=2000.0, seed=4)
    scenes = []
    offsets = [(15, 10), (12, 14), (20, 6), (9, 16), (17, 3), (22, 9)]
    for k in range(24):
        a, b = offsets[k % len(offsets)]
        extra = [(a + 3, 0)] if k % 3 == 0 else ([(-(a + 2), 0)] if k % 3 == 1 else [])
        scenes.append([(0, 0), (a, -b), (a, b)] + extra)
    x, y = [], []
    for k, sc in enumerate(scenes):
        cx, cy = 80 + 140 * (k % 6), 80 + 140 * (k // 6)
        for dx, dy in sc:
            x.append(cx + dx)
            y.append(cy + dy)
    n = len(x)
    ag, pt = initial_state(prm, n, 1, seed=1)
    ag["x"][:] = np.array(x, np.float32)
    ag["y"][:] = np.array(y, np.float32)
    ag["theta"][:] = 0.0
    ag["override_mode"][:] = -1
    pt["x"][:], pt["y"][:] = 930.0, 930.0
    sim = ForagingSim(prm, agents=ag, patches=pt)
    a0, p0 = sim.agents_numpy(), sim.patches_numpy()
    sim.step()
    fp, ip, s = prm.oracle_arrays()
    a1, p1, soc, failed = oracle.forage_step(a0, p0, fp, ip, s)
    _check(sim.agents_numpy(), sim.patches_numpy(), sim.soc_numpy(), a1, p1,
           soc.astype(np.uint8), f"rv {rv}")
    diag = sim.diag.cpu().numpy()
    assert int(np.sum(a1["override_mode"] == 4)) >= 40
    assert diag[5] >= 8, diag        # FP64 bearings (neighbours exactly ahead / behind)
    if rv % 2 == 0:
        assert diag[6] >= 4, diag    # pairwise-sum replays (mirror ties)
