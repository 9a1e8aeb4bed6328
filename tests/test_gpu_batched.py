"""GPU tests of the batched sweep (abm_vpf_flock_batched / abm_gb300.batched).

Each instance of a batched step must be bit-identical to the plain step of that instance alone
(same kernels, same decisions), including per-instance ALP0/BET0 and multi-step runs through a
captured CUDA graph; small instances are also checked against the oracle.
"""
import numpy as np
import pytest

import oracle
from conftest import gpu_available
from _gpu_helpers import check_vpf

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def _instances(seed=4):
    from abm_gb300.batched import sweep_instances
    inst = sweep_instances(n_instances=7, n_min=10, n_max=300, alp_grid=(3, 3), seed=seed,
                           width=600.0, height=600.0)
    inst[0] = {k: (v[:1] if isinstance(v, np.ndarray) else v) for k, v in inst[0].items()}
    rng = np.random.default_rng(seed)
    for d in inst:
        d["v"] = rng.uniform(0, 1, len(d["x"])).astype(np.float32)
    return inst


def test_batched_step_matches_single_instances():
    from abm_gb300.batched import BatchedSweep
    from abm_gb300.params import VFParams
    from abm_gb300.swarm import VFSwarm
    vp = VFParams(alp1=0.08, bet1=0.08, width=600.0, height=600.0, rv=1200)
    inst = _instances()
    b = BatchedSweep(vp, inst)
    b.step(want_vpf=True, want_terms=True)
    bv, bt = b.vpf_numpy(), b.terms.cpu().numpy()
    for k, d in enumerate(inst):
        a0, a1 = int(b.offsets[k]), int(b.offsets[k + 1])
        n = a1 - a0
        s = VFSwarm(vp, d["x"], d["y"], d["theta"], d["v"], alp0=np.full(n, d["alp0"]),
                    bet0=np.full(n, d["bet0"]))
        s.step(want_vpf=True, want_terms=True)
        assert np.array_equal(s.vpf_numpy(), bv[a0:a1]), k
        assert np.array_equal(s.terms.cpu().numpy(), bt[a0:a1]), k
        st = s.state_numpy()
        bs = b.instance_state(k)
        for key in st:
            assert np.array_equal(st[key], bs[key]), (k, key)


def test_batched_group_and_l1_forms_agree():
    """The group form (8 consecutive entries of the schedule per warp, straddling instances)
    and the L1 form give identical results for a sweep, also with a schedule that interleaves
    the instances' agents."""
    import torch
    from abm_gb300 import _lib
    from abm_gb300.batched import BatchedSweep
    from abm_gb300.params import VFParams
    lib = _lib.load()
    vp = VFParams(alp1=0.08, bet1=0.08, width=600.0, height=600.0, rv=1200)
    inst = _instances(seed=21)
    outs = []
    try:
        for mode, shuffle in ((1, False), (3, False), (3, True)):
            _lib.check(lib.abm_vpf_set_step_mode(mode, 1))
            b = BatchedSweep(vp, inst)
            if shuffle:   # a schedule whose groups of 8 mix agents of several instances
                perm = np.random.default_rng(2).permutation(b.n).astype(np.int32)
                b.order = torch.as_tensor(perm, device="cuda")
            b.step(want_vpf=True, want_terms=True)
            outs.append((b.vpf_numpy(), b.terms.cpu().numpy(), b.state_numpy()))
    finally:
        lib.abm_vpf_set_step_mode(0, 1)
    for o in outs[1:]:
        assert np.array_equal(o[0], outs[0][0])
        assert np.array_equal(o[1], outs[0][1])
        for k in o[2]:
            assert np.array_equal(o[2][k], outs[0][2][k])


def test_batched_small_instances_vs_oracle():
    from abm_gb300.batched import BatchedSweep
    from abm_gb300.params import VFParams
    vp = VFParams(alp1=0.08, bet1=0.08, width=600.0, height=600.0, rv=1200)
    inst = _instances(seed=9)[:4]
    b = BatchedSweep(vp, inst)
    b.step(want_vpf=True, want_terms=True)
    bv, bt = b.vpf_numpy(), b.terms.cpu().numpy()
    for k, d in enumerate(inst):
        a0, a1 = int(b.offsets[k]), int(b.offsets[k + 1])
        p = dict(vp.oracle_dict(), alp0=d["alp0"], bet0=d["bet0"])
        st = {key: np.asarray(d[key], np.float64) for key in ("x", "y", "theta", "v")}
        ref = oracle.vf_step(st, p, want_excuse=True)
        check_vpf(bv[a0:a1], ref["vpf"], ref["excuse"], ref["near"], k)
        scale = np.maximum(np.abs(ref["terms"]), 1e-6)
        assert np.all(np.abs(bt[a0:a1] - ref["terms"]) / scale <= 1e-5), k


def test_batched_sweep_step_vs_oracle_every_instance():
    """One step of the 512-instance sweep (N per instance uniform in [10, 500], ALP0 and BET0
    on a 16 x 32 grid over [0.1, 3], Rv=1200, 1000 x 1000 walls), every instance against the
    oracle's step from the same state: VPF (excuse mask only), the six terms within 1e-5
    relative, the new state within 2 float32 ulps."""
    from abm_gb300.batched import BatchedSweep, sweep_instances
    from abm_gb300.params import VFParams
    vp = VFParams(gam=0.1, v0=1.0, alp1=0.08, bet1=0.08, width=1000.0, height=1000.0,
                  rv=1200, radius=10.0)
    inst = sweep_instances(n_instances=512, seed=3)
    rng = np.random.default_rng(31)
    for d in inst:   # moving agents, so the update's speed terms are exercised too
        d["v"] = rng.uniform(0, 1.5, len(d["x"])).astype(np.float32)
    b = BatchedSweep(vp, inst)
    b.step(want_vpf=True, want_terms=True)
    bv, bt = b.vpf_numpy(), b.terms.cpu().numpy()
    tot_px = tot_near = 0
    for k, d in enumerate(inst):
        a0, a1 = int(b.offsets[k]), int(b.offsets[k + 1])
        # the sweep passes ALP0 / BET0 to the kernels as float32 per-agent values
        p = dict(vp.oracle_dict(), alp0=float(np.float32(d["alp0"])),
                 bet0=float(np.float32(d["bet0"])))
        st = {key: np.asarray(d[key], np.float32).astype(np.float64)
              for key in ("x", "y", "theta", "v")}
        ref = oracle.vf_step(st, p, want_excuse=True)
        px, _, near = check_vpf(bv[a0:a1], ref["vpf"], ref["excuse"], ref["near"], k)
        tot_px += px
        tot_near += near
        scale = np.maximum(np.abs(ref["terms"]), 1e-6)
        err = np.abs(bt[a0:a1] - ref["terms"]) / scale
        assert np.all(err <= 1e-5), (k, float(err.max()))
        new = b.instance_state(k)
        for key in ("x", "y", "theta", "v"):
            r32 = ref[key].astype(np.float32)
            ulp = np.spacing(np.abs(r32)).astype(np.float64)
            diff = np.abs(new[key].astype(np.float64) - ref[key])
            assert np.all(diff <= 2 * ulp + 1e-12), (k, key, float((diff / ulp).max()))
    print(f"sweep: {b.n} agents, {tot_px} mismatched pixels, {tot_near} near-boundary pairs")


def test_batched_torus_far_agents_forms_agree():
    """Batched instances on a 600 x 600 torus with agents far outside it (x = 1500, -1300,
    1e9; y = 1400): the group kernel takes their offsets through the double-float path and
    equals the L1 form bit for bit (VPF, terms, new state), with and without direct phase B."""
    from abm_gb300 import _lib
    from abm_gb300.batched import BatchedSweep, sweep_instances
    from abm_gb300.params import VFParams
    lib = _lib.load()
    inst = sweep_instances(n_instances=6, n_min=20, n_max=90, alp_grid=(2, 3), seed=51,
                           width=600.0, height=600.0)
    far = [(1500.0, 100.0), (-1300.0, 200.0), (1.0e9, 300.0), (100.0, 1400.0)]
    for k, d in enumerate(inst[:4]):
        d["x"][k % len(d["x"])] = np.float32(far[k][0])
        d["y"][k % len(d["y"])] = np.float32(far[k][1])
    outs = []
    try:
        for rv in (1200, 200):   # the arena within the cull radius (direct phase B) or not
            vp = VFParams(alp1=0.08, bet1=0.08, width=600.0, height=600.0, rv=rv,
                          boundary="infinite")
            for mode in (1, 3):
                _lib.check(lib.abm_vpf_set_step_mode(mode, 1))
                b = BatchedSweep(vp, inst)
                b.step(want_vpf=True, want_terms=True)
                outs.append((rv, b.vpf_numpy(), b.terms.cpu().numpy(), b.state_numpy()))
    finally:
        lib.abm_vpf_set_step_mode(0, 1)
    for a, b in ((outs[0], outs[1]), (outs[2], outs[3])):
        assert np.array_equal(a[1], b[1]), a[0]
        assert np.array_equal(a[2], b[2]), a[0]
        for k in a[3]:
            assert np.array_equal(a[3][k], b[3][k]), (a[0], k)


@pytest.mark.parametrize("fov_ratio", [0.5, 1.0])
def test_batched_torus_sweep_vs_oracle_every_instance(fov_ratio):
    """A sweep shaped like the reference's torus experiments: 121 instances of N=10 on an
    11 x 11 (ALP0, BET0) grid, a 900 x 900 torus, R = 5.5, field of view +-fov_ratio * pi with
    Rv = 600 / fov_ratio (the metarunner's rescaling).  Rv = 1200 takes phase B straight from
    the scan, Rv = 600 the compaction queue.  Every instance against the oracle's step from
    the same state: VPF (excuse mask only), terms within 1e-5 relative, state within 2 ulps."""
    import math
    from abm_gb300.batched import BatchedSweep, sweep_instances
    from abm_gb300.params import VFParams
    rv = int(600 / fov_ratio)
    vp = VFParams(alp1=0.08, bet1=0.08, width=900.0, height=900.0, rv=rv, radius=5.5,
                  boundary="infinite", fov=(-fov_ratio * math.pi, fov_ratio * math.pi))
    inst = sweep_instances(n_instances=121, n_min=10, n_max=10, alp_grid=(11, 11),
                           alp_range=(0.0, 5.0), width=900.0, height=900.0, radius=5.5,
                           seed=41)
    rng = np.random.default_rng(41)
    for d in inst:
        d["v"] = rng.uniform(0, 1.5, len(d["x"])).astype(np.float32)
    b = BatchedSweep(vp, inst)
    b.step(want_vpf=True, want_terms=True)
    bv, bt = b.vpf_numpy(), b.terms.cpu().numpy()
    for k, d in enumerate(inst):
        a0, a1 = int(b.offsets[k]), int(b.offsets[k + 1])
        p = dict(vp.oracle_dict(), alp0=float(np.float32(d["alp0"])),
                 bet0=float(np.float32(d["bet0"])))
        st = {key: np.asarray(d[key], np.float32).astype(np.float64)
              for key in ("x", "y", "theta", "v")}
        ref = oracle.vf_step(st, p, want_excuse=True)
        check_vpf(bv[a0:a1], ref["vpf"], ref["excuse"], ref["near"], k)
        scale = np.maximum(np.abs(ref["terms"]), 1e-6)
        err = np.abs(bt[a0:a1] - ref["terms"]) / scale
        assert np.all(err <= 1e-5), (k, float(err.max()))
        new = b.instance_state(k)
        for key in ("x", "y", "theta", "v"):
            r32 = ref[key].astype(np.float32)
            ulp = np.spacing(np.abs(r32)).astype(np.float64)
            diff = np.abs(new[key].astype(np.float64) - ref[key])
            assert np.all(diff <= 2 * ulp + 1e-12), (k, key, float((diff / ulp).max()))


def test_batched_graph_run_matches_eager_steps():
    from abm_gb300.batched import BatchedSweep
    from abm_gb300.params import VFParams
    vp = VFParams(alp1=0.08, bet1=0.08, width=600.0, height=600.0, rv=1200)
    inst = _instances(seed=11)
    g = BatchedSweep(vp, inst)
    e = BatchedSweep(vp, inst)
    g.run(24, chunk=10)          # 2 graph replays + 4 single steps
    for _ in range(24):
        e.step()
    sg, se = g.state_numpy(), e.state_numpy()
    for key in sg:
        assert np.array_equal(sg[key], se[key]), key


def test_polarisation_statistic_on_device():
    """The on-device polarisation series equals |sum (cos, sin)| / N of each instance's state
    after every step (numpy, FP64), in eager steps and in replayed graphs alike."""
    from abm_gb300.batched import BatchedSweep
    from abm_gb300.params import VFParams
    vp = VFParams(alp1=0.08, bet1=0.08, width=600.0, height=600.0, rv=400)
    inst = _instances(seed=13)
    a, b = BatchedSweep(vp, inst), BatchedSweep(vp, inst)
    a.track_polarisation(300)
    b.track_polarisation(300)
    want = []
    for _ in range(120):
        a.step()
        row = []
        for k in range(len(inst)):
            th = a.instance_state(k)["theta"].astype(np.float64)
            row.append(np.hypot(np.cos(th).sum(), np.sin(th).sum()) / len(th))
        want.append(row)
    pa = a.polarisation()
    assert pa.shape == (len(inst), 120)
    assert np.max(np.abs(pa - np.array(want).T)) < 1e-6
    b.run(120, chunk=100)
    assert np.array_equal(b.polarisation(), pa)


@pytest.mark.parametrize("boundary", ["walls", "infinite"])
@pytest.mark.parametrize("width,fov", [(600.0, None), (600.0, (-1.5, 2.0)), (3000.0, None),
                                       (3000.0, (-1.5, 2.0))])
def test_batched_group_kernel_forms_agree(width, fov, boundary):
    """The batched group kernel's forms -- phase B straight from the scan (every offset inside
    the cull radius) or through the compaction queue (a larger arena), each with the full
    field of view or a partial one, between walls and on the torus (minimal images) -- against
    the L1 form on the same sweep: VPF, terms and new state bit-identical."""
    import math
    from abm_gb300 import _lib
    from abm_gb300.batched import BatchedSweep, sweep_instances
    from abm_gb300.params import VFParams
    lib = _lib.load()
    kw = {} if fov is None else {"fov": fov}
    vp = VFParams(alp1=0.08, bet1=0.08, width=width, height=width, rv=1200, boundary=boundary,
                  **kw)
    inst = sweep_instances(n_instances=9, n_min=10, n_max=260, alp_grid=(3, 3), seed=31,
                           width=width, height=width)
    cull = 10.0 / math.tan(2 * math.pi / 1200)   # h >= 1 only within this distance (R = 10)
    ext2 = 2 * width * width if boundary == "walls" else width * width / 2
    assert (ext2 <= cull * cull) == (width < 1000.0)
    outs = []
    try:
        for mode in (1, 3):
            _lib.check(lib.abm_vpf_set_step_mode(mode, 1))
            b = BatchedSweep(vp, inst)
            for _ in range(2):
                b.step(want_vpf=True, want_terms=True)
            outs.append((b.vpf_numpy(), b.terms.cpu().numpy(), b.state_numpy()))
    finally:
        lib.abm_vpf_set_step_mode(0, 1)
    assert np.array_equal(outs[0][0], outs[1][0])
    assert np.array_equal(outs[0][1], outs[1][1])
    for k in outs[0][2]:
        assert np.array_equal(outs[0][2][k], outs[1][2][k]), k
