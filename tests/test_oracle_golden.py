"""Pin the CPU oracle against fixtures produced by the reference itself.

The fixtures come from tests/golden/make_golden.py, which runs the reference's own
vf_supcalc / VFAgent / Agent code; the known-answer vectors are the reference's own
(abm/projects/cooperative_signaling/cs_agent/tests/test_cs_supcalc.py:143-169).
Discrete outputs (VPF pixels, projection rows) must match exactly; FP64 scalars within a
few ulps (1e-12 relative), since numpy's BLAS dot and SIMD cos may round differently.
"""
import numpy as np
import pytest

import oracle
from conftest import load_cases, GOLDEN


def test_known_answer_projection_field():
    z = np.load(GOLDEN + "/known_answers.npz")
    # test_cs_supcalc.py:143-158: Rv=8, position (-1,-1), R=1, orientation 0, object (0,-1)
    expected = np.array([[0., 0., 0., 0., 1., 1., 0., 0.]])
    assert np.array_equal(z["pf_rv8"], expected)
    assert np.array_equal(z["pf_rv8_sizes"], expected)
    out = oracle.projection_field((-np.pi, np.pi), 8, [-1, -1], 1, 0, [[0, -1]])
    assert np.array_equal(out, expected)
    out = oracle.projection_field((-np.pi, np.pi), 8, [-1, -1], 1, 0, [[0, -1]], [1])
    assert np.array_equal(out, expected)


def test_known_answer_closed_angle():
    z = np.load(GOLDEN + "/known_answers.npz")
    # test_cs_supcalc.py:161-169
    assert np.allclose(z["ca_out"], [0.0, -np.pi / 2, -np.pi])
    for v1, v2, exp in zip(z["ca_v1"], z["ca_v2"], z["ca_out"]):
        assert oracle.calculate_closed_angle(v1, v2) == exp


@pytest.mark.parametrize("rv", sorted(set(range(8, 5001, 97)) | {61, 122, 197, 1200, 2666, 3600}))
def test_arange_and_linspace_match_numpy(rv):
    assert np.array_equal(oracle.arange_phi(rv), np.arange(-np.pi, np.pi, 2 * np.pi / rv))
    assert np.array_equal(oracle.linspace(rv), np.linspace(-np.pi, np.pi, rv))


def test_arange_length_quirk_all_rv():
    bad = [rv for rv in range(8, 5001)
           if len(np.arange(-np.pi, np.pi, 2 * np.pi / rv)) != rv]
    assert len(bad) == len([rv for rv in range(8, 5001) if len(oracle.arange_phi(rv)) != rv])
    assert 61 in bad and 1200 not in bad and 3600 not in bad


def test_projection_field_matches_reference():
    cases = load_cases("projection")
    assert len(cases) == 48
    for c in cases:
        rv, n = int(c["rv"]), int(c["n"])
        sizes = c["sizes"] if c["sizes"].size else None
        vr = None if np.isnan(c["vr"]) else float(c["vr"])
        out = oracle.projection_field(tuple(c["fov"]), rv, c["pos"], float(c["R"]), float(c["ori"]),
                                      c["objs"], sizes,
                                      "infinite" if int(c["boundary"]) else "walls",
                                      float(c["W"]), float(c["H"]), vr)
        ref = np.unpackbits(c["out"], axis=1)[:, :rv]
        assert out.shape == (n, rv)
        assert np.array_equal(out.astype(np.uint8), ref)


def test_vswrm_matches_reference():
    cases = load_cases("vswrm")
    for c in cases:
        rv = int(c["rv"])
        phi = np.arange(-np.pi, np.pi, 2 * np.pi / rv)
        V = c["V"].astype(np.float64)
        assert np.array_equal(oracle.dphi_v(V), c["dphi"])
        prm = dict(zip(["gam", "v0", "alp0", "alp1", "alp2", "bet0", "bet1", "bet2"], c["prm"]))
        full = {k: 0.0 for k in oracle.P_FIELDS}
        full.update(prm)
        out = oracle.vswrm(float(c["vel"]), phi, V, full)
        ref = c["out"]
        scale = np.max(np.abs(ref)) + 1e-300
        assert np.allclose(out, ref, rtol=1e-12, atol=1e-12 * scale), (rv, out, ref)


def _params(vec):
    return dict(zip(oracle.P_FIELDS, vec))


def test_snapshot_steps_match_reference():
    cases = load_cases("steps")
    for c in cases:
        p = _params(c["params"])
        rv = int(p["rv"])
        st = {k: c[k] for k in ("x", "y", "theta", "v")}
        opt = lambda a: a if a.size else None
        out = oracle.vf_step(st, p, radii=c["radii"], alp0=opt(c["alp0"]), bet0=opt(c["bet0"]),
                             v0=opt(c["v0"]))
        ref_vpf = np.unpackbits(c["vpf"], axis=1)[:, :rv]
        assert np.array_equal(out["vpf"], ref_vpf), c["name"]
        assert np.allclose(out["terms"], c["terms"], rtol=1e-12, atol=1e-12), c["name"]
        for k in ("x", "y", "theta", "v"):
            assert np.allclose(out[k], c[k + "_new"], rtol=1e-12, atol=1e-9), (c["name"], k)
        assert out["phi_mismatch"] == (str(c["name"]) == "mismatch_rv61")


def test_sequential_steps_match_reference():
    for c in load_cases("sequential"):
        p = _params(c["params"])
        traj = c["traj"]
        st = dict(zip(("x", "y", "theta", "v"), traj[0]))
        for t in range(1, traj.shape[0]):
            out = oracle.vf_step(st, p, radii=c["radii"], sequential=True, want_vpf=False)
            for q, k in enumerate(("x", "y", "theta", "v")):
                assert np.allclose(out[k], traj[t][q], rtol=1e-11, atol=1e-8), (t, k)
            st = {k: out[k] for k in ("x", "y", "theta", "v")}


def test_social_channel_matches_reference():
    for c in load_cases("social"):
        rv = int(c["rv"])
        n = len(c["x"])
        radii = np.full(n, float(c["R"]))
        ref = np.unpackbits(c["out"], axis=1)[:, :rv]
        for i in range(n):
            out = oracle.social_vpf(i, c["x"], c["y"], radii, c["theta"], c["exploit"],
                                    c["patch"], float(c["vr"]), bool(c["vex"]), bool(c["pw"]),
                                    rv, tuple(c["fov"]))
            assert np.array_equal(out > 0, ref[i] > 0), (i,)
