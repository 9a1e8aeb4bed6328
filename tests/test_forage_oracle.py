"""CPU checks of the foraging oracle (oracle.forage_step) against fixtures produced by the
reference's own foraging step (tests/golden/make_forage_golden.py), and of the Philox-4x32-10
generator (oracle and library host function) against the generator's published
known-answer vectors."""
import ctypes

import numpy as np
import pytest

import oracle
from conftest import load_cases

# Philox-4x32-10 known-answer vectors (Random123 kat_vectors): (counter, key, output)
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,want", PHILOX_KAT)
def test_philox_known_answers(ctr, key, want):
    assert tuple(oracle.philox4x32(ctr, key)) == want
    from abm_gb300 import _lib
    lib = _lib.load()
    out = (ctypes.c_uint32 * 4)()
    lib.abm_philox4x32((ctypes.c_uint32 * 4)(*ctr), (ctypes.c_uint32 * 2)(*key), out)
    assert tuple(out) == want


AGENT_INT = ("mode", "override_mode", "env_status", "env_status_before", "pool_success",
             "patch_id", "novelty")


def _ulps32(a, b):
    """Distance in float32 units in the last place, relative to the larger magnitude."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = np.spacing(np.maximum(np.abs(a), np.abs(b)).astype(np.float32)).astype(np.float64)
    return np.abs(a - b) / np.maximum(scale, np.spacing(np.float32(1.0)))


def test_forage_oracle_matches_reference():
    cases = load_cases("forage")
    assert len(cases) >= 12
    for ci, c in enumerate(cases):
        ag = {k[3:]: v for k, v in c.items() if k.startswith("in_")}
        pt = {k[4:]: v for k, v in c.items() if k.startswith("pin_")}
        a, p, soc, failed = oracle.forage_step(ag, pt, c["fp"], c["ip"], 0, c["uniforms"])
        rv = int(c["ip"][7])
        want_soc = np.unpackbits(c["soc"], axis=1)[:, :rv]
        assert np.array_equal(soc.astype(np.uint8), want_soc), ci
        for k in AGENT_INT:
            assert np.array_equal(a[k].astype(np.int64), c["out_" + k]), (ci, k)
        for k in ("w", "u", "collected", "collected_before"):
            np.testing.assert_allclose(a[k], c["out_" + k], rtol=0, atol=1e-12,
                                       err_msg=f"case {ci} {k}")
        for k in ("x", "y", "theta", "v"):
            assert np.max(_ulps32(a[k], c["out_" + k])) <= 2.0, (ci, k)
        assert np.array_equal(p["left"], c["pout_left"]), ci
        assert np.array_equal(p["id"], c["pout_id"]), ci
        assert failed == 0


def test_forage_oracle_branches_covered():
    """The fixtures reach the branches that matter: exploiting agents, random walks,
    relocations, emptied patches and teleports."""
    cases = load_cases("forage")
    modes = np.concatenate([c["out_mode"] for c in cases])
    assert {0, 1, 2} <= set(modes.tolist())
    emptied = sum(int(np.sum(c["pout_id"] < 0)) for c in cases)
    assert emptied >= 2
    notified = sum(int(np.sum(c["out_env_status"] == 1)) for c in cases)
    assert notified >= 5


def test_forage_params_from_env_and_round_trip():
    """.env keys of abm/app.py and the -1 maxima of sims.py:176-179; the oracle arrays and the
    C struct carry the same values."""
    import math
    from abm_gb300.foraging import ForageParams
    env = {"N": "10", "MIN_RESOURCE_PER_PATCH": "100", "MAX_RESOURCE_PER_PATCH": "-1",
           "MIN_RESOURCE_QUALITY": "0.25", "MAX_RESOURCE_QUALITY": "-1", "AGENT_FOV": "0.5",
           "VISION_RANGE": "2000", "POOLING_TIME": "0", "TELEPORT_TO_MIDDLE": "0",
           "DEC_TW": "0.4", "MOV_REL_TH_MAX": "0.7", "VISUAL_FIELD_RESOLUTION": "320"}
    p = ForageParams.from_env(env, seed=3)
    assert (p.min_resc_units, p.max_resc_units) == (100, 101)
    assert (p.min_resc_quality, p.max_resc_quality) == (0.25, 0.25)
    assert p.T_w == 0.4 and p.reloc_theta_max == 0.7 and p.rv == 320 and not p.teleport_exploit
    fp, ip, seed = p.oracle_arrays()
    assert ForageParams.from_arrays(fp, ip, seed) == p
    c = p.to_c()
    assert c.fov0 == -0.5 * math.pi and c.fov1 == 0.5 * math.pi and c.seed == 3
    assert c.min_resc_units == 100 and c.max_resc_units == 101 and c.T_w == 0.4
    env.update({"AGENT_AGENT_COLLISION": "1", "GHOST_WHILE_EXPLOIT": "0"})
    q = ForageParams.from_env(env)
    assert q.collide_agents and not q.ghost_mode
    fp, ip, seed = q.oracle_arrays()
    assert len(ip) == 12 and ip[10] == 1 and ip[11] == 0
    assert ForageParams.from_arrays(fp, ip, seed) == q
    # arrays written before the collision switches existed: collisions off
    assert not ForageParams.from_arrays(fp, ip[:10], seed).collide_agents


def test_forage_params_struct_layout():
    """The ctypes mirror of abm_forage_params has the C layout: the library's defaults land in
    the right fields, up to the last one, and equal ForageParams' defaults."""
    import ctypes
    from abm_gb300 import _lib
    from abm_gb300.foraging import ForageParams
    lib = _lib.load()
    c = _lib.AbmForageParams()
    ctypes.memset(ctypes.byref(c), 0x7F, ctypes.sizeof(c))
    assert lib.abm_forage_params_default(ctypes.byref(c)) == 0
    d = ForageParams().to_c()
    for name, _ in _lib.AbmForageParams._fields_:
        assert getattr(c, name) == getattr(d, name), name
    assert (c.rv, c.seed, c.collide_agents, c.ghost_mode) == (1200, 0, 0, 1)


def test_np_mean_restatement_matches_numpy():
    """The oracle's pairwise-summation mean equals np.mean bit for bit, on random vectors and
    on the proximity fields' value patterns (0, 1 and one weight) seen through flipped views."""
    rng = np.random.default_rng(11)
    for _ in range(300):
        n = int(rng.integers(1, 5000))
        a = rng.standard_normal(n) * np.exp(rng.uniform(-30, 30, n))
        assert oracle.np_mean(a) == np.mean(a)
        w = 1 - rng.uniform(0, 45) / rng.choice([30.0, 150.0, 2000.0])
        f = np.flip(rng.choice([0.0, 1.0, w], n, p=[0.6, 0.1, 0.3]))
        h = n // 2
        for v in (f[:h], f[h:]):
            if len(v):
                assert oracle.np_mean(np.ascontiguousarray(v)) == np.mean(v)


def test_collision_oracle_matches_reference():
    """Foraging steps with agent-agent collisions: the oracle against the reference's own
    collision block (Simulation.agent_agent_collision_proximity with Agent.projection_field
    and the collided-agent bookkeeping of sims.py:735-784) followed by its step."""
    cases = load_cases("collision")
    assert len(cases) >= 16
    for ci, c in enumerate(cases):
        assert int(c["ip"][10]) == 1
        ag = {k[3:]: v for k, v in c.items() if k.startswith("in_")}
        pt = {k[4:]: v for k, v in c.items() if k.startswith("pin_")}
        a, p, soc, failed = oracle.forage_step(ag, pt, c["fp"], c["ip"], 0, c["uniforms"])
        rv = int(c["ip"][7])
        assert np.array_equal(soc.astype(np.uint8), np.unpackbits(c["soc"], axis=1)[:, :rv]), ci
        for k in AGENT_INT:
            assert np.array_equal(a[k].astype(np.int64), c["out_" + k]), (ci, k)
        for k in ("w", "u", "collected", "collected_before"):
            np.testing.assert_allclose(a[k], c["out_" + k], rtol=0, atol=1e-12,
                                       err_msg=f"case {ci} {k}")
        for k in ("x", "y", "theta", "v"):
            assert np.max(_ulps32(a[k], c["out_" + k])) <= 2.0, (ci, k)
        assert np.array_equal(p["left"], c["pout_left"]), ci


def test_collision_fixtures_cover_the_branches():
    """The collision fixtures reach: agents left in collide mode, collide mode ended, stopped
    agents (front occupied), both ghost settings, both teleport settings, odd and small Rv
    (front slice from a negative start), a vision range below the proximity radius (negative
    field weight), and several manoeuvres of one agent in a step."""
    cases = load_cases("collision")
    ip = np.array([c["ip"] for c in cases])
    assert set(ip[:, 11]) == {0, 1} and set(ip[:, 2]) == {0, 1}
    assert {120, 121} <= set(ip[:, 7].tolist())
    assert any(float(c["fp"][29]) < 40 for c in cases)
    out_mode = np.concatenate([c["out_override_mode"] for c in cases])
    in_mode = np.concatenate([c["in_override_mode"] for c in cases])
    assert np.sum(out_mode == 4) >= 20
    assert np.sum((in_mode == 4) & (out_mode != 4)) >= 5
    stopped = np.concatenate([(c["out_override_mode"] == 4) & (c["out_v"] == 0) for c in cases])
    assert stopped.sum() >= 5
    assert sum(int(c["pairs"]) for c in cases) >= 200
