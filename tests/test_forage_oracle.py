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
