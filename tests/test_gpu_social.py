"""GPU parity of the foraging social channel (abm_vpf_social_fields) against the reference
(fixtures from Agent.calc_social_V_proj itself) and against the oracle on seeded foraging
swarms (N=100, Rv=1200, 3 patches): fields bit-exact."""
import math

import numpy as np
import pytest

import oracle
from conftest import load_cases, gpu_available

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def test_social_fields_golden():
    from abm_gb300.forage import social_fields
    for c in load_cases("social"):
        rv = int(c["rv"])
        out = social_fields(c["x"], c["y"], c["theta"], c["exploit"], c["patch"], float(c["vr"]),
                            bool(c["vex"]), bool(c["pw"]), rv, tuple(c["fov"]), float(c["R"]))
        ref = np.unpackbits(c["out"], axis=1)[:, :rv]
        assert np.array_equal(out, ref)


@pytest.mark.parametrize("seed,vr,vex,pw,fov", [
    (1, 200.0, True, True, (-math.pi, math.pi)),
    (2, 1000.0, True, False, (-math.pi, math.pi)),
    (3, 3000.0, False, True, (-math.pi, math.pi)),
    (4, 400.0, True, True, (-0.6 * math.pi, 0.6 * math.pi)),
    (5, 150.0, True, True, (-0.45 * math.pi, 0.45 * math.pi)),
])
def test_social_fields_vs_oracle(seed, vr, vex, pw, fov):
    from abm_gb300.forage import social_fields
    rng = np.random.default_rng(seed)
    n, W, R, rv = 100, 1000.0, 10.0, 1200
    x = rng.uniform(20, 20 + W, n).astype(np.float32)
    y = rng.uniform(20, 20 + W, n).astype(np.float32)
    # a few tight clusters (agents on patches) so occlusion and trimming matter
    for p in range(3):
        c = rng.uniform(100, W - 100, 2)
        idx = rng.choice(n, 12, replace=False)
        x[idx] = (c[0] + rng.normal(0, 25, 12)).astype(np.float32)
        y[idx] = (c[1] + rng.normal(0, 25, 12)).astype(np.float32)
    th = rng.uniform(0, 2 * np.pi, n).astype(np.float32)
    exploit = (rng.random(n) < 0.3).astype(np.int32)
    patch = np.where(exploit > 0, rng.integers(-1, 3, n), -1).astype(np.int32)
    out = social_fields(x, y, th, exploit, patch, vr, vex, pw, rv, fov, R)
    radii = np.full(n, R)
    for i in range(n):
        ref = oracle.social_vpf(i, x.astype(np.float64), y.astype(np.float64), radii,
                                th.astype(np.float64), exploit, patch, vr, vex, pw, rv, fov)
        assert np.array_equal(out[i], (ref > 0).astype(np.uint8)), i
