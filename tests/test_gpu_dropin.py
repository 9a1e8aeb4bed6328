"""GPU parity of the drop-in twins of the reference's math module (abm_gb300.vf_supcalc)
against fixtures produced by the reference itself (tests/golden/make_golden.py):

* projection_field (vf_supcalc.py:20-138): rows bit-exact, except the pixels that an object
  whose edge angle is within 1e-9 rad of a pixel / width boundary flips under its alternative
  decisions (the oracle's per-object excuse rows; counted);
* VSWRM_flocking_state_variables (vf_supcalc.py:161-254): within 1e-5 relative.
"""
import numpy as np
import pytest

import oracle
from conftest import load_cases, gpu_available

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def test_projection_field_golden():
    from abm_gb300 import vf_supcalc
    excused = 0
    for c in load_cases("projection"):
        rv, n = int(c["rv"]), int(c["n"])
        sizes = c["sizes"] if c["sizes"].size else None
        vr = None if np.isnan(c["vr"]) else float(c["vr"])
        bc = "infinite" if int(c["boundary"]) else "walls"
        out = vf_supcalc.projection_field(tuple(c["fov"]), rv, c["pos"], float(c["R"]),
                                          float(c["ori"]), c["objs"], sizes, bc,
                                          float(c["W"]), float(c["H"]), vr)
        ref = np.unpackbits(c["out"], axis=1)[:, :rv]
        assert out.shape == (n, rv) and out.dtype == np.float64
        ex, near = oracle.projection_excuse(tuple(c["fov"]), rv, c["pos"], float(c["R"]),
                                            float(c["ori"]), c["objs"], sizes, bc,
                                            float(c["W"]), float(c["H"]), vr)
        for r in range(n):
            bad = out[r].astype(np.uint8) != ref[r]
            if bad.any():
                assert near[r] and np.all(ex[r][bad]), (r, np.where(bad)[0][:8])
                excused += 1
    assert excused <= 2


def test_projection_field_known_answer():
    """test_cs_supcalc.py:143-158 known answer, through the GPU drop-in."""
    from abm_gb300 import vf_supcalc
    out = vf_supcalc.projection_field((-np.pi, np.pi), 8, np.array([-1, -1]), 1, 0,
                                      [np.array([0, -1])], None)
    assert np.array_equal(out, [[0., 0., 0., 0., 1., 1., 0., 0.]])


def test_vswrm_golden():
    from abm_gb300 import vf_supcalc

    class P:
        pass

    for c in load_cases("vswrm"):
        rv = int(c["rv"])
        phi = np.arange(-np.pi, np.pi, 2 * np.pi / rv)
        prm = P()
        for k, v in zip(["GAM", "V0", "ALP0", "ALP1", "ALP2", "BET0", "BET1", "BET2"], c["prm"]):
            setattr(prm, k, float(v))
        V = c["V"].astype(np.float64)
        out = vf_supcalc.VSWRM_flocking_state_variables(float(c["vel"]), phi, V, prm,
                                                        verbose=True)
        ref = c["out"]
        scale = np.maximum(np.abs(ref), 1e-6)
        assert np.all(np.abs(np.array(out) - ref) / scale <= 1e-5), (rv, out, ref)
        dv, dpsi = vf_supcalc.VSWRM_flocking_state_variables(float(c["vel"]), phi, V, prm)
        assert abs(dv - out[0]) <= 1e-12 and abs(dpsi - out[1]) <= 1e-12


def test_vswrm_length_mismatch_raises_like_numpy():
    from abm_gb300 import vf_supcalc

    class P:
        GAM, V0, ALP0, ALP1, ALP2, BET0, BET1, BET2 = 0.1, 1.0, 1.0, 0.08, 0.0, 1.0, 0.08, 0.0

    phi = np.arange(-np.pi, np.pi, 2 * np.pi / 61)      # 62 entries for Rv = 61
    with pytest.raises(ValueError):
        vf_supcalc.VSWRM_flocking_state_variables(0.0, phi, np.zeros(61), P())


@pytest.mark.parametrize("pinned", [True, False])
def test_flock_step_host_matches_device_step(pinned):
    """abm_vpf_flock_step_host on host state (page-locked: gathered / written by the kernels;
    pageable: copied by the driver) gives the device step's result, over several steps."""
    import torch
    from abm_gb300 import _lib
    from abm_gb300.params import VFParams
    from abm_gb300.swarm import VFSwarm, step_host
    from _gpu_helpers import seeded_swarm
    lib = _lib.load()
    st = seeded_swarm(17, 900, 1500.0, 1500.0, R=5.0)
    vp = VFParams(width=1500.0, height=1500.0, rv=1000, radius=5.0)
    sw = VFSwarm(vp, st["x"], st["y"], st["theta"], st["v"])
    f32 = lambda a: np.ascontiguousarray(a, dtype=np.float32)
    mk = (lambda a: torch.from_numpy(f32(a)).pin_memory()) if pinned else \
        (lambda a: torch.from_numpy(f32(a).copy()))
    h_in = {k: mk(st[k]) for k in ("x", "y", "theta", "v")}
    h_out = {k: mk(np.zeros_like(st[k])) for k in ("x", "y", "theta", "v")}
    s = torch.cuda.current_stream()
    cp = vp.to_c()
    for _ in range(3):
        sw.step()
        step_host(lib, cp, len(st["x"]), h_in, h_out, s)
        h_in, h_out = h_out, h_in
    torch.cuda.synchronize()
    want = sw.state_numpy()
    for k in want:
        assert np.array_equal(h_in[k].numpy(), want[k]), k
