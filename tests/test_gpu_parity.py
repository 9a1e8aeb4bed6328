"""GPU parity of the fused flock step (abm_vpf_flock_step) against the reference.

Against the golden fixtures (produced by the reference itself) and against the FP64 oracle
on seeded swarms.  Bars (from the specification of this path):
* VPF bits: bit-exact, except the pixels that pairs whose edge angle lies within 1e-9 rad of a
  pixel / width boundary flip under their alternative decisions (the oracle's excuse mask;
  never a whole row); mismatches and near-boundary pairs are counted and reported.
* VSWRM integrals (dvel, dpsi and the four terms): within 1e-5 relative.
* New state: the FP64 update rounded to float32: within 2 float32 ulps of the reference.
"""
import numpy as np
import pytest

import oracle
from conftest import load_cases, gpu_available
from _gpu_helpers import seeded_swarm, check_vpf

pytestmark = pytest.mark.gpu

TERM_RTOL = 1e-5


def _swarm_from(state, p, radii=None, alp0=None, bet0=None, v0=None):
    from abm_gb300.swarm import VFSwarm
    from abm_gb300.params import VFParams
    vp = VFParams(gam=p["gam"], v0=p["v0"], alp0=p["alp0"], alp1=p["alp1"], alp2=p["alp2"],
                  bet0=p["bet0"], bet1=p["bet1"], bet2=p["bet2"],
                  boundary="infinite" if p["boundary"] else "walls",
                  limit_movement=bool(p["limit_movement"]), max_vel=p["max_vel"],
                  max_th=p["max_th"], width=p["width"], height=p["height"],
                  window_pad=p["window_pad"], fov=(p["fov0"], p["fov1"]), rv=int(p["rv"]),
                  radius=p["radius"], dt=p["dt"])
    return VFSwarm(vp, state["x"], state["y"], state["theta"], state["v"], radius=radii,
                   alp0=alp0, bet0=bet0, v0=v0)


def _check_terms(gpu, ref, what):
    scale = np.maximum(np.abs(ref), 1e-6)
    err = np.abs(gpu - ref) / scale
    assert np.all(err <= TERM_RTOL), (what, float(err.max()))


def _check_state(gpu, ref, what):
    for k in ("x", "y", "theta", "v"):
        r32 = ref[k].astype(np.float32)
        ulp = np.spacing(np.abs(r32)).astype(np.float64)
        diff = np.abs(gpu[k].astype(np.float64) - ref[k])
        assert np.all(diff <= 2 * ulp + 1e-12), (what, k, float((diff / ulp).max()))


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def test_golden_steps():
    for c in load_cases("steps"):
        p = dict(zip(oracle.P_FIELDS, c["params"]))
        rv = int(p["rv"])
        opt = lambda a: a if a.size else None
        hetero = bool(np.any(c["radii"] != c["radii"][0]))
        st = {k: c[k] for k in ("x", "y", "theta", "v")}
        sw = _swarm_from(st, p, c["radii"] if hetero else None, opt(c["alp0"]), opt(c["bet0"]),
                         opt(c["v0"]))
        status = sw.step(want_vpf=True, want_terms=True)
        name = str(c["name"])
        assert status == (1 if name == "mismatch_rv61" else 0), name
        ref_vpf = np.unpackbits(c["vpf"], axis=1)[:, :rv]
        gpu_vpf = sw.vpf_numpy()
        orc = oracle.vf_step(st, p, radii=c["radii"], alp0=opt(c["alp0"]), bet0=opt(c["bet0"]),
                             v0=opt(c["v0"]), want_excuse=True)
        # against the reference's own VPF (fixture) and against the oracle's
        check_vpf(gpu_vpf, ref_vpf, orc["excuse"], orc["near"], name)
        check_vpf(gpu_vpf, orc["vpf"], orc["excuse"], orc["near"], name)
        terms = sw.terms.cpu().numpy()
        _check_terms(terms, c["terms"], name)
        new = sw.state_numpy()
        _check_state(new, {k: c[k + "_new"] for k in ("x", "y", "theta", "v")}, name)


@pytest.mark.parametrize("seed,n,rv,R,W,boundary,kappa", [
    (1, 2, 8, 10.0, 500.0, 0, None),
    (2, 3, 64, 10.0, 500.0, 0, None),
    (3, 10, 1200, 10.0, 500.0, 0, None),
    (4, 100, 1200, 10.0, 1000.0, 0, None),
    (5, 100, 1200, 10.0, 300.0, 1, None),
    (6, 300, 3600, 5.0, 5000.0, 0, 2.0),
    (7, 257, 3600, 5.0, 800.0, 1, 2.0),
    (8, 64, 333, 7.0, 200.0, 0, None),
])
def test_seeded_parity_vs_oracle(seed, n, rv, R, W, boundary, kappa):
    p = dict(gam=0.1, v0=1.0, alp0=1.0, alp1=0.08, alp2=0.0, bet0=1.0, bet1=0.08, bet2=0.0,
             boundary=boundary, limit_movement=0, max_vel=3.0, max_th=0.1, width=W, height=W,
             window_pad=30.0, fov0=-np.pi, fov1=np.pi, rv=rv, radius=R, dt=1.0)
    st = seeded_swarm(seed, n, W, W, R=R, kappa=kappa)
    sw = _swarm_from(st, p)
    sw.step(want_vpf=True, want_terms=True)
    orc = oracle.vf_step(st, p, want_excuse=True)
    px, rows, near = check_vpf(sw.vpf_numpy(), orc["vpf"], orc["excuse"], orc["near"],
                               (seed, n, rv))
    print(f"seed {seed}: {px} mismatched pixels in {rows} agents, {near} near-boundary pairs")
    _check_terms(sw.terms.cpu().numpy(), orc["terms"], (seed, n, rv))
    _check_state(sw.state_numpy(), orc, (seed, n, rv))
    d = sw.diagnostics()
    assert d["timeouts"] == 0 and d["nonfinite"] == 0


def test_full_size_all_agents_cfg2():
    """N=4096, Rv=3600, R=5 in 5000x5000 (the large-swarm workload), every agent against the
    oracle's step from the same snapshot: VPF (excuse mask only), the six VSWRM terms within
    1e-5 relative and the new state within 2 float32 ulps."""
    n, rv, R, W = 4096, 3600, 5.0, 5000.0
    p = dict(gam=0.1, v0=1.0, alp0=1.0, alp1=0.08, alp2=0.0, bet0=1.0, bet1=0.08, bet2=0.0,
             boundary=0, limit_movement=0, max_vel=3.0, max_th=0.1, width=W, height=W,
             window_pad=30.0, fov0=-np.pi, fov1=np.pi, rv=rv, radius=R, dt=1.0)
    st = seeded_swarm(42, n, W, W, R=R, kappa=2.0)
    sw = _swarm_from(st, p)
    sw.step(want_vpf=True, want_terms=True)
    orc = oracle.vf_step(st, p, want_excuse=True)
    px, rows, near = check_vpf(sw.vpf_numpy(), orc["vpf"], orc["excuse"], orc["near"], "cfg2")
    d = sw.diagnostics()
    print(f"cfg2: {px} mismatched pixels in {rows} agents; near-boundary pairs: oracle {near}, "
          f"kernel {d['near_boundary']} (of {d['pairs_resolved']} re-decided)")
    _check_terms(sw.terms.cpu().numpy(), orc["terms"], "cfg2")
    _check_state(sw.state_numpy(), orc, "cfg2")
    assert d["timeouts"] == 0 and d["nonfinite"] == 0


def test_max_size_spot_check_tiled():
    """The largest sizes: N=17000 agents (above 16384, so the automatic choice is the tiled
    form with TMA-staged, double-buffered neighbour tiles) and Rv=16384 (the maximum), R=3 in
    12000x12000; 4 focal agents recomputed by the oracle (union of the rows, no dense
    materialisation)."""
    n, rv, R, W = 17000, 16384, 3.0, 12000.0
    p = dict(gam=0.1, v0=1.0, alp0=1.0, alp1=0.08, alp2=0.0, bet0=1.0, bet1=0.08, bet2=0.0,
             boundary=0, limit_movement=0, max_vel=3.0, max_th=0.1, width=W, height=W,
             window_pad=30.0, fov0=-np.pi, fov1=np.pi, rv=rv, radius=R, dt=1.0)
    st = seeded_swarm(77, n, W, W, R=R, kappa=None)
    sw = _swarm_from(st, p)
    sw.step(want_vpf=True, want_terms=True)
    terms = sw.terms.cpu().numpy()
    d = sw.diagnostics()
    assert d["timeouts"] == 0 and d["nonfinite"] == 0
    rng = np.random.default_rng(1)
    phi = oracle.arange_phi(rv)
    for i in rng.choice(n, 4, replace=False):
        words = sw.vpf_bits[i].cpu().numpy().view(np.uint32)
        gpu = np.unpackbits(words.view(np.uint8), bitorder="little")[:rv]
        objs = np.stack([np.delete(st["x"], i), np.delete(st["y"], i)], axis=1)
        V, _, ex, near = oracle.projection_union((-np.pi, np.pi), rv, [st["x"][i], st["y"][i]],
                                                 R, st["theta"][i], objs, want_excuse=True)
        check_vpf(gpu, V.astype(np.uint8), ex, near, ("tiled", i))
        ref = oracle.vswrm(st["v"][i], phi, V, p)
        _check_terms(terms[i], ref, i)


def test_permutation_invariance_full_size():
    """The VPF is a union of intervals: reordering the agents must permute the outputs
    exactly (N=4096, Rv=3600)."""
    from abm_gb300.params import VFParams
    from abm_gb300.swarm import VFSwarm
    n, W = 4096, 5000.0
    st = seeded_swarm(11, n, W, W, R=5.0, kappa=2.0)
    vp = VFParams(alp1=0.08, bet1=0.08, width=W, height=W, rv=3600, radius=5.0)
    a = VFSwarm(vp, st["x"], st["y"], st["theta"], st["v"])
    a.step(want_vpf=True, want_terms=True)
    perm = np.random.default_rng(3).permutation(n)
    b = VFSwarm(vp, st["x"][perm], st["y"][perm], st["theta"][perm], st["v"][perm])
    b.step(want_vpf=True, want_terms=True)
    assert np.array_equal(a.vpf_numpy()[perm], b.vpf_numpy())
    assert np.array_equal(a.terms.cpu().numpy()[perm], b.terms.cpu().numpy())
    sa, sb = a.state_numpy(), b.state_numpy()
    for k in sa:
        assert np.array_equal(sa[k][perm], sb[k])


def _configs_agree(vp, st, configs, radius=None):
    from abm_gb300 import _lib
    from abm_gb300.swarm import VFSwarm
    lib = _lib.load()
    outs = []
    try:
        for mode, wpa, warps, tile, split in configs:
            _lib.check(lib.abm_vpf_set_step_mode(mode, wpa))
            _lib.check(lib.abm_vpf_set_step_config(warps, tile))
            _lib.check(lib.abm_vpf_set_step_split(split))
            s = VFSwarm(vp, st["x"], st["y"], st["theta"], st["v"], radius=radius)
            s.step(want_vpf=True, want_terms=True)
            outs.append((s.vpf_numpy(), s.terms.cpu().numpy(), s.state_numpy()))
    finally:
        lib.abm_vpf_set_step_mode(0, 1)
        lib.abm_vpf_set_step_config(8, 8192)
        lib.abm_vpf_set_step_split(0)
    for o in outs[1:]:
        assert np.array_equal(o[0], outs[0][0])
        assert np.array_equal(o[1], outs[0][1])
        for k in o[2]:
            assert np.array_equal(o[2][k], outs[0][2][k])


def test_launch_configs_agree():
    """Every kernel form and launch configuration gives bit-identical results: the L1 form
    with 1, 2 and 4 warps per agent, one block per agent or the neighbours split over 2-16
    blocks (partial bitmasks OR-ed in the workspace, integrals in the finish kernel), the
    group form (one warp for 4 agents) with 1-16 chunks, and the TMA-tiled form with several
    (warps per block, tile) shapes including multi-tile double buffering."""
    from abm_gb300.params import VFParams
    st = seeded_swarm(5, 1000, 2000.0, 2000.0, R=5.0)
    vp = VFParams(width=2000.0, height=2000.0, rv=1200, radius=5.0)
    _configs_agree(vp, st, ((1, 1, 8, 8192, 1), (1, 2, 8, 8192, 1), (1, 4, 8, 8192, 1),
                            (1, 1, 8, 8192, 2), (1, 1, 8, 8192, 4), (1, 1, 8, 8192, 16),
                            (1, 2, 8, 8192, 8), (1, 4, 8, 8192, 4), (0, 1, 8, 8192, 0),
                            (3, 1, 8, 8192, 1), (3, 1, 8, 8192, 2), (3, 1, 8, 8192, 8),
                            (3, 1, 8, 8192, 16),
                            (2, 1, 8, 2048, 0), (2, 1, 4, 256, 0), (2, 1, 16, 1024, 0),
                            (2, 1, 32, 64, 0), (2, 1, 1, 4096, 0)))


def test_group_form_partial_last_group():
    """1003 agents (a last group of 3) and a swarm of 3 (one partial group): the group form
    with and without chunks equals the L1 form."""
    from abm_gb300.params import VFParams
    for n, W in ((1003, 2000.0), (3, 200.0)):
        st = seeded_swarm(15, n, W, W, R=5.0)
        vp = VFParams(width=W, height=W, rv=1200, radius=5.0)
        _configs_agree(vp, st, ((1, 1, 8, 8192, 1), (3, 1, 8, 8192, 1), (3, 1, 8, 8192, 4)))


def test_group_chunk_plan_agrees():
    """Swarms whose automatic group form spans more than one wave of blocks take the
    decreasing round-major chunk plan (4096 agents: 8 rounds; 5003 agents: 4 rounds and a last
    group of 3): bit-identical to the unsplit group form and to the L1 form."""
    from abm_gb300.params import VFParams
    for n, W in ((4096, 5000.0), (5003, 5000.0)):
        st = seeded_swarm(21, n, W, W, R=5.0, kappa=2.0)
        vp = VFParams(width=W, height=W, rv=3600, radius=5.0)
        _configs_agree(vp, st, ((0, 1, 8, 8192, 0), (3, 1, 8, 8192, 1), (3, 1, 8, 8192, 4),
                                (1, 1, 8, 8192, 4)))


def test_launch_configs_agree_torus_radii():
    """The same agreement on the infinite (torus) arena with per-agent radii."""
    from abm_gb300.params import VFParams
    st = seeded_swarm(8, 700, 1500.0, 1500.0, R=5.0)
    radius = np.random.default_rng(8).uniform(3.0, 9.0, 700).astype(np.float32)
    vp = VFParams(width=1500.0, height=1500.0, rv=2000, radius=5.0, boundary="infinite")
    _configs_agree(vp, st, ((1, 1, 8, 8192, 1), (1, 1, 8, 8192, 4), (1, 2, 8, 8192, 16),
                            (2, 1, 8, 1024, 0)), radius=radius)


@pytest.mark.parametrize("fov", [None, (-1.5, 2.0)])
def test_group_form_torus_agrees(fov):
    """The group form on the torus (equal radii) against the L1 and tiled forms, bit for bit:
    a random swarm on a 1000 x 800 torus plus agents placed on the wrap seam (offsets of
    exactly W/2 and H/2, and offsets W/2 +- 1e-5 whose float32 difference rounds to W/2, on
    either side), two agents whose images coincide, and agents more than 2W or 2H from others,
    one of them at x = 1e9 (the double-float offset's path)."""
    from abm_gb300.params import VFParams
    st = seeded_swarm(31, 1200, 1000.0, 800.0, pad=10.0, R=5.0)
    seam = [(-1e-5, 200.0), (500.0, 210.0), (1e-5, 220.0), (100.0, 230.0), (600.0, 240.0),
            (20.0, -1e-5), (30.0, 400.0), (40.0, 1e-5), (50.0, 50.0), (60.0, 450.0),
            (0.0, 0.0), (1000.0, 0.0), (2600.0, 300.0), (300.0, 2000.0), (-2300.0, 500.0),
            (1.0e9, 100.0)]
    rng = np.random.default_rng(31)
    for k in ("x", "y"):
        extra = np.array([p[0 if k == "x" else 1] for p in seam], dtype=np.float32)
        st[k] = np.concatenate([st[k], extra])
    m = len(seam)
    st["theta"] = np.concatenate([st["theta"],
                                  rng.uniform(0, 2 * np.pi, m).astype(np.float32)])
    st["v"] = np.concatenate([st["v"], rng.uniform(0, 1.5, m).astype(np.float32)])
    kw = {} if fov is None else {"fov": fov}
    vp = VFParams(width=1000.0, height=800.0, rv=1200, radius=5.0, boundary="infinite", **kw)
    _configs_agree(vp, st, ((1, 1, 8, 8192, 1), (3, 1, 8, 8192, 1), (3, 1, 8, 8192, 4),
                            (0, 1, 8, 8192, 0), (1, 1, 8, 8192, 4), (2, 1, 8, 1024, 0)))


def test_group_form_torus_needs_float_extent():
    """A torus whose width is not exact in float32 is refused by the group form (the
    automatic configuration then takes the L1 form)."""
    from abm_gb300 import _lib
    from abm_gb300.params import VFParams
    from abm_gb300.swarm import VFSwarm
    lib = _lib.load()
    st = seeded_swarm(32, 200, 1000.0, 1000.0, pad=10.0, R=5.0)
    vp = VFParams(width=1000.1, height=1000.0, rv=1200, radius=5.0, boundary="infinite")
    try:
        _lib.check(lib.abm_vpf_set_step_mode(3, 1))
        s = VFSwarm(vp, st["x"], st["y"], st["theta"], st["v"])
        with pytest.raises(Exception, match="group form"):
            s.step()
    finally:
        lib.abm_vpf_set_step_mode(0, 1)
    _configs_agree(vp, st, ((0, 1, 8, 8192, 0), (1, 1, 8, 8192, 1)))


def test_split_workspace_is_clean_between_calls():
    """The split form's per-agent bitmasks in the stream workspace are zero again after every
    step: swarms of different sizes and Rv stepped one after another on one stream give the
    same results as each stepped first."""
    from abm_gb300 import _lib
    from abm_gb300.params import VFParams
    from abm_gb300.swarm import VFSwarm
    lib = _lib.load()
    cases = [(seeded_swarm(11, 900, 1800.0, 1800.0, R=5.0), VFParams(width=1800.0, height=1800.0,
                                                                    rv=1200, radius=5.0)),
             (seeded_swarm(12, 300, 900.0, 900.0, R=5.0), VFParams(width=900.0, height=900.0,
                                                                  rv=3600, radius=5.0)),
             (seeded_swarm(13, 1500, 2500.0, 2500.0, R=5.0), VFParams(width=2500.0,
                                                                     height=2500.0, rv=640,
                                                                     radius=5.0))]

    def run(st, vp):
        s = VFSwarm(vp, st["x"], st["y"], st["theta"], st["v"])
        s.step(want_vpf=True, want_terms=True)
        return s.vpf_numpy(), s.terms.cpu().numpy(), s.state_numpy()

    try:
        _lib.check(lib.abm_vpf_set_step_split(4))
        first = [run(*c) for c in cases]
        again = [run(*c) for c in reversed(cases)][::-1]
    finally:
        lib.abm_vpf_set_step_split(0)
    for a, b in zip(first, again):
        assert np.array_equal(a[0], b[0])
        assert np.array_equal(a[1], b[1])
        for k in a[2]:
            assert np.array_equal(a[2][k], b[2][k])


def test_double_float_sincos():
    """The FP32-only double-float cos/sin of the focal heading is within 1e-13 of FP64."""
    import ctypes
    import torch
    from abm_gb300 import _lib
    lib = _lib.load()
    rng = np.random.default_rng(1)
    th = np.concatenate([rng.uniform(0, 2 * np.pi, 200000), rng.uniform(-7, 14, 20000),
                         np.arange(0, 1025) * (2 * np.pi / 1024)]).astype(np.float32)
    t = torch.as_tensor(th, device="cuda")
    out = torch.empty((len(th), 2), dtype=torch.float64, device="cuda")
    _lib.check(lib.abm_vpf_check_sincos(_lib.fptr(t), len(th), _lib.dptr(out), None))
    o = out.cpu().numpy()
    th64 = th.astype(np.float64)
    assert np.max(np.abs(o[:, 0] - np.cos(th64))) < 1e-13
    assert np.max(np.abs(o[:, 1] - np.sin(th64))) < 1e-13


def test_unaligned_state_uses_plain_loads():
    """State arrays that are not 16-byte aligned take the non-TMA staging path; results are
    identical to the aligned path."""
    import torch
    from abm_gb300.params import VFParams
    from abm_gb300.swarm import VFSwarm
    from abm_gb300 import _lib
    lib = _lib.load()
    st = seeded_swarm(9, 777, 1500.0, 1500.0)
    vp = VFParams(width=1500.0, height=1500.0, rv=1200)
    try:
        _lib.check(lib.abm_vpf_set_step_mode(2, 0))
        _lib.check(lib.abm_vpf_set_step_config(8, 256))
        a = VFSwarm(vp, st["x"], st["y"], st["theta"], st["v"])
        a.step(want_vpf=True)
        b = VFSwarm(vp, st["x"], st["y"], st["theta"], st["v"])
        for k in ("x", "y"):
            big = torch.zeros(b.n + 1, dtype=torch.float32, device="cuda")
            big[1:] = b._cur[k]
            b._cur[k] = big[1:]          # 4-byte offset: not 16-byte aligned
        b.step(want_vpf=True)
    finally:
        lib.abm_vpf_set_step_mode(0, 1)
        lib.abm_vpf_set_step_config(8, 8192)
    assert np.array_equal(a.vpf_numpy(), b.vpf_numpy())


def test_polarisation_ensemble_cfg0():
    """Long runs diverge per trajectory (float32 state); compare the ensemble mean
    polarisation (data_loader.py:1818-1824) of 48 seeds x 300 steps of the N=10 walls
    workload between the GPU and the oracle's snapshot dynamics."""
    from abm_gb300.params import VFParams
    from abm_gb300.swarm import VFSwarm
    n, steps, seeds = 10, 300, 48
    p = dict(gam=0.1, v0=1.0, alp0=1.0, alp1=0.08, alp2=0.0, bet0=1.0, bet1=0.08, bet2=0.0,
             boundary=0, limit_movement=0, max_vel=3.0, max_th=0.1, width=500.0,
             height=500.0, window_pad=30.0, fov0=-np.pi, fov1=np.pi, rv=1200, radius=10.0,
             dt=1.0)
    vp = VFParams(alp1=0.08, bet1=0.08, width=500.0, height=500.0, rv=1200)
    pol_g, pol_o = [], []
    for seed in range(seeds):
        st = seeded_swarm(100 + seed, n, 500.0, 500.0, vmax=0.0)
        sw = VFSwarm(vp, st["x"], st["y"], st["theta"], st["v"])
        o = dict(st)
        for t in range(steps):
            sw.step()
            o = oracle.vf_step(o, p, want_vpf=False, want_terms=False)
        g = sw.state_numpy()
        pol = lambda th: np.hypot(np.cos(th).sum(), np.sin(th).sum()) / n
        pol_g.append(pol(g["theta"].astype(np.float64)))
        pol_o.append(pol(o["theta"]))
    pol_g, pol_o = np.array(pol_g), np.array(pol_o)
    se = np.sqrt(pol_g.var() / seeds + pol_o.var() / seeds)
    assert abs(pol_g.mean() - pol_o.mean()) < 4 * se + 1e-3, (pol_g.mean(), pol_o.mean(), se)


@pytest.mark.parametrize("boundary", [0, 1])
def test_single_agent_and_empty_swarm(boundary):
    """A lone agent sees nothing (empty VPF, zero integrals) and still moves like the oracle's
    update; a swarm of zero agents is a valid no-op of the step and of the recorder."""
    import ctypes
    import torch
    from abm_gb300 import _lib
    p = dict(gam=0.1, v0=1.0, alp0=1.0, alp1=0.08, alp2=0.0, bet0=1.0, bet1=0.08, bet2=0.0,
             boundary=boundary, limit_movement=0, max_vel=3.0, max_th=0.1, width=500.0,
             height=500.0, window_pad=30.0, fov0=-np.pi, fov1=np.pi, rv=1200, radius=10.0,
             dt=1.0)
    st = {"x": np.array([21.0]), "y": np.array([263.5]), "theta": np.array([3.0]),
          "v": np.array([0.75])}
    sw = _swarm_from(st, p)
    o = st
    for _ in range(12):   # reaches the left wall / seam
        sw.step(want_vpf=True, want_terms=True)
        ref = oracle.vf_step(o, p)
        assert not sw.vpf_numpy().any()
        _check_terms(sw.terms.cpu().numpy(), ref["terms"], "single")
        _check_state(sw.state_numpy(), ref, "single")
        o = {k: sw.state_numpy()[k].astype(np.float64) for k in ("x", "y", "theta", "v")}
    lib = _lib.load()
    empty = _lib.AbmSwarmState(None, None, None, None)
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    assert lib.abm_vpf_flock_step(ctypes.byref(empty), ctypes.byref(empty), 0,
                                  ctypes.byref(sw._cparams), None, None, None, None, s) >= 0
    step = torch.zeros(2, dtype=torch.int32, device="cuda")
    rec = _lib.AbmVfRecording(4, _lib.i32ptr(step), None, None, None, None, None)
    assert lib.abm_vpf_record(ctypes.byref(empty), 0, None, 1200, ctypes.byref(rec), s) == 0
    torch.cuda.synchronize()
    assert step.tolist() == [1, 0]
