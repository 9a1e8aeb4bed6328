"""Generate the golden fixtures in this directory by running the REFERENCE implementation.

Run from the repository root in a container that has the reference checkout:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_golden.py /path/to/reference

The reference (scioip34/ABM 1.2.0) is pure Python; four import shims let its hot-path
modules load without python-dotenv, pygame, matplotlib (used only for agent colours) or
scipy.integrate.trapz (removed from recent SciPy; np.trapezoid applies the same trapezoid
rule).  The reference is never modified.

Fixtures (all inputs are FP32-representable so the CUDA path sees the identical state):

* known_answers.npz   the reference's own known-answer vectors
                      (cs_agent/tests/test_cs_supcalc.py:143-169) run through the VF twins
* projection.npz      single-focal vf_supcalc.projection_field calls (vf_supcalc.py:20-138)
* vswrm.npz           VSWRM_flocking_state_variables(verbose=True) on chosen/random fields
* steps.npz           one snapshot step of whole swarms through VFAgent.calc_soc_v_proj,
                      perform_action and the boundary rule (vf_agent.py:52-77, :216-309)
* sequential.npz      a few pygame-order (Gauss-Seidel) steps of small swarms
* social.npz          Agent.calc_social_V_proj foraging channel with occlusion (agent.py:396-603)
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def install_shims(ref_root: str):
    sys.dont_write_bytecode = True
    d = types.ModuleType("dotenv")
    d.dotenv_values = lambda *a, **k: {}
    sys.modules["dotenv"] = d
    pg = types.ModuleType("pygame")
    sp = types.ModuleType("pygame.sprite")

    class Sprite:  # only the base class is needed
        def __init__(self, *a, **k):
            pass

    sp.Sprite = Sprite
    pg.sprite = sp
    sys.modules["pygame"] = pg
    sys.modules["pygame.sprite"] = sp
    mpl = types.ModuleType("matplotlib")      # vf_agent.py:1 imports it for colours only
    sys.modules["matplotlib"] = mpl
    import scipy.integrate as si
    si.trapz = lambda y, x=None, dx=1.0, axis=-1: np.trapezoid(y, x=x, dx=dx, axis=axis)
    sys.path.insert(0, ref_root)


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


class Params:
    def __init__(self, **kw):
        self.__dict__.update(kw)


def base_params(**over):
    p = dict(gam=0.1, v0=1.0, alp0=1.0, alp1=0.08, alp2=0.0, bet0=1.0, bet1=0.08, bet2=0.0,
             boundary=0, limit_movement=0, max_vel=3.0, max_th=0.1, width=500.0, height=500.0,
             window_pad=30.0, fov0=-np.pi, fov1=np.pi, rv=1200, radius=10.0, dt=1.0)
    p.update(over)
    return p


def params_vec(p):
    from oracle import P_FIELDS  # the same slot order the oracle uses
    return np.array([float(p[k]) for k in P_FIELDS], np.float64)


def make_vfagents(VFAgent, p, x, y, th, v, radii, alp0=None, bet0=None, v0=None):
    ags = []
    for i in range(len(x)):
        a = object.__new__(VFAgent)
        a.id = i
        a.position = np.array([x[i], y[i]], dtype=np.float64)
        a.radius = float(radii[i])
        a.orientation = float(th[i])
        a.velocity = float(v[i])
        a.v_field_res = int(p["rv"])
        a.FOV = (p["fov0"], p["fov1"])
        a.boundary_cond = "infinite" if p["boundary"] else "walls"
        a.WIDTH, a.HEIGHT = p["width"], p["height"]
        a.window_pad = p["window_pad"]
        a.boundaries_x = [a.window_pad, a.window_pad + a.WIDTH]
        a.boundaries_y = [a.window_pad, a.window_pad + a.HEIGHT]
        a.limit_movement = bool(p["limit_movement"])
        a.max_vel, a.max_th = p["max_vel"], p["max_th"]
        a.PHI = np.arange(-np.pi, np.pi, (2 * np.pi) / a.v_field_res)
        a.ALP0 = None if alp0 is None else float(alp0[i])
        a.BET0 = None if bet0 is None else float(bet0[i])
        a.V0 = None if v0 is None else float(v0[i])
        a.verbose_supcalc = True
        a.lines = []
        a.is_moved_with_cursor = 0
        a.agent_state = "flocking"
        a.dv = a.dphi = a.ablob = a.aedge = a.bblob = a.bedge = 0.0
        ags.append(a)
    return ags


def ref_step(mods, p, state, radii, alp0=None, bet0=None, v0=None, sequential=False):
    """One reference step; returns new state, raw-order VPFs (n x Rv) and 6 terms."""
    VFAgent, vf_params = mods
    vf_params.GAM, vf_params.V0 = p["gam"], p["v0"]
    vf_params.ALP0, vf_params.ALP1, vf_params.ALP2 = p["alp0"], p["alp1"], p["alp2"]
    vf_params.BET0, vf_params.BET1, vf_params.BET2 = p["bet0"], p["bet1"], p["bet2"]
    x, y, th, v = (state[k] for k in ("x", "y", "theta", "v"))
    n = len(x)
    live = make_vfagents(VFAgent, p, x, y, th, v, radii, alp0, bet0, v0)
    frozen = make_vfagents(VFAgent, p, x, y, th, v, radii, alp0, bet0, v0)
    vpf = np.zeros((n, int(p["rv"])), np.uint8)
    terms = np.zeros((n, 6))
    import contextlib
    import io
    for i, a in enumerate(live):
        field = a.calc_soc_v_proj(live if sequential else frozen)
        a.soc_v_field = field
        vpf[i] = np.flip(field) > 0
        with contextlib.redirect_stdout(io.StringIO()):
            a.perform_action()
        if a.boundary_cond == "walls":
            a.reflect_from_walls()
        else:
            a.teleport_infinite_arena()
        if len(a.PHI) == len(a.soc_v_field):
            terms[i] = [a.dv, a.dphi, a.ablob, a.aedge, a.bblob, a.bedge]
    new = {"x": np.array([a.position[0] for a in live], np.float64),
           "y": np.array([a.position[1] for a in live], np.float64),
           "theta": np.array([a.orientation for a in live], np.float64),
           "v": np.array([a.velocity for a in live], np.float64)}
    return new, vpf, terms


def swarm(rng, n, W, H, pad, R, kappa=None):
    x = f32(rng.uniform(pad - R, pad + W - R, n))
    y = f32(rng.uniform(pad - R, pad + H - R, n))
    if kappa is None:
        th = f32(rng.uniform(0, 2 * np.pi, n))
    else:
        th = f32(np.mod(rng.vonmises(rng.uniform(0, 2 * np.pi), kappa, n), 2 * np.pi))
    v = f32(rng.uniform(0, 1.5, n))
    return {"x": x, "y": y, "theta": th, "v": v}


def main(ref_root):
    install_shims(ref_root)
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from abm.projects.visual_flocking.vf_agent import vf_supcalc as vs
    from abm.projects.visual_flocking.vf_agent.vf_agent import VFAgent
    from abm.projects.visual_flocking.vf_contrib import vf_params
    from abm.agent.agent import Agent
    rng = np.random.default_rng(20261203)

    # ---------------------------------------------------------------- known answers
    ka = {}
    ka["pf_rv8"] = vs.projection_field((-np.pi, np.pi), 8, np.array([-1, -1]), 1, 0,
                                       [np.array([0, -1])], None)
    ka["pf_rv8_sizes"] = vs.projection_field((-np.pi, np.pi), 8, np.array([-1, -1]), 1, 0,
                                             [np.array([0, -1])], [1])
    ka["ca_v1"] = np.array([[1, 0], [1, 0], [1, 0]], np.float64)
    ka["ca_v2"] = np.array([[1, 0], [0, 1], [-1, 0]], np.float64)
    ka["ca_out"] = np.array([vs.calculate_closed_angle(np.array(a), np.array(b))
                             for a, b in zip(ka["ca_v1"], ka["ca_v2"])])
    np.savez_compressed(os.path.join(HERE, "known_answers.npz"), **ka)

    # ---------------------------------------------------------------- projection_field
    pcs = []
    specs = []
    for rv in (8, 64, 1200, 3600):
        for boundary in ("walls", "infinite"):
            for k in range(6):
                specs.append((rv, boundary, k))
    for (rv, boundary, k) in specs:
        W = H = float(rng.choice([500.0, 1000.0, 5000.0]))
        R = float(rng.choice([1.0, 5.0, 10.0]))
        n = int(rng.integers(1, 24))
        pos = f32(rng.uniform(0, W, 2))
        objs = f32(rng.uniform(0, W, (n, 2)))
        if k == 0:   # close neighbours (wide projections, wraps)
            objs = f32(pos + rng.uniform(-4 * R, 4 * R, (n, 2)))
        if k == 1:   # coincident, straight ahead/behind/left/right
            objs[0] = pos
            if n > 4:
                objs[1] = f32(pos + [3 * R, 0]); objs[2] = f32(pos + [-3 * R, 0])
                objs[3] = f32(pos + [0, 3 * R]); objs[4] = f32(pos + [0, -3 * R])
        sizes = f32(rng.choice([1.0, 5.0, 10.0], n)) if k == 2 else None
        fov = (-np.pi, np.pi) if k != 3 else (-0.45 * np.pi, 0.45 * np.pi)
        ori = float(f32(rng.uniform(0, 2 * np.pi))) if k != 1 else float(
            rng.choice([0.0, np.float32(np.pi / 2), np.float32(np.pi)]))
        vr = None if k != 4 else float(rng.uniform(50, W))
        out = vs.projection_field(fov, rv, np.array(pos), R, ori, [np.array(o) for o in objs],
                                  None if sizes is None else list(sizes), boundary_cond=boundary,
                                  arena_width=W, arena_height=H, vision_range=vr)
        pcs.append(dict(rv=rv, boundary=1 if boundary == "infinite" else 0, W=W, H=H, R=R,
                        pos=pos, objs=objs, sizes=np.zeros(0) if sizes is None else sizes,
                        fov=np.array(fov), ori=ori, vr=np.nan if vr is None else vr,
                        out=np.packbits(out.astype(np.uint8), axis=1), n=n))
    np.savez_compressed(os.path.join(HERE, "projection.npz"),
                        **{f"c{i}_{k}": np.asarray(v) for i, c in enumerate(pcs)
                           for k, v in c.items()}, count=len(pcs))

    # ---------------------------------------------------------------- VSWRM
    vcs = []
    for rv in (8, 64, 1200, 3600, 61):
        Phi = np.arange(-np.pi, np.pi, (2 * np.pi) / rv)
        n = len(Phi)
        pats = [np.zeros(n), np.ones(n)]
        b = np.zeros(n); b[n // 4: n // 2] = 1; pats.append(b)
        b = np.zeros(n); b[:3] = 1; b[-2:] = 1; pats.append(b)             # wrap blob
        b = np.zeros(n); b[0] = 1; b[n // 3: n // 3 + 2] = 1; pats.append(b)  # V0=1,V-1=0
        b = np.zeros(n); b[-1] = 1; b[5 % n] = 1; pats.append(b)            # V-1=1,V0=0
        for _ in range(4):
            pats.append((rng.random(n) < rng.uniform(0.05, 0.9)).astype(np.float64))
        for V in pats:
            vel = float(f32(rng.uniform(0, 2)))
            prm = Params(GAM=0.1, V0=1.0, ALP0=float(f32(rng.uniform(0.1, 3))), ALP1=0.08,
                         ALP2=0.0, BET0=float(f32(rng.uniform(0.1, 3))), BET1=0.08, BET2=0.0)
            out = vs.VSWRM_flocking_state_variables(vel, Phi, V, prm, verbose=True)
            vcs.append(dict(rv=rv, V=V.astype(np.uint8), vel=vel,
                            prm=np.array([prm.GAM, prm.V0, prm.ALP0, prm.ALP1, prm.ALP2,
                                          prm.BET0, prm.BET1, prm.BET2]),
                            out=np.array(out, np.float64), dphi=vs.dPhi_V_of(Phi, V)))
    np.savez_compressed(os.path.join(HERE, "vswrm.npz"),
                        **{f"c{i}_{k}": np.asarray(v) for i, c in enumerate(vcs)
                           for k, v in c.items()}, count=len(vcs))

    # ---------------------------------------------------------------- snapshot steps
    mods = (VFAgent, vf_params)
    scs = []
    step_specs = [
        dict(name="cfg0_walls_n10", n=10, p=base_params()),
        dict(name="n2", n=2, p=base_params(rv=64)),
        dict(name="n3_rv8", n=3, p=base_params(rv=8)),
        dict(name="n100_rv1200", n=100, p=base_params(width=1000.0, height=1000.0)),
        dict(name="n40_rv3600_r5", n=40, p=base_params(rv=3600, radius=5.0, width=5000.0,
                                                      height=5000.0), kappa=2.0),
        dict(name="torus_n30", n=30, p=base_params(boundary=1, width=400.0, height=300.0)),
        dict(name="limit_n20", n=20, p=base_params(limit_movement=1, max_vel=1.2, max_th=0.05)),
        dict(name="hetero_n16", n=16, p=base_params(), hetero=True),
        dict(name="fov_n20", n=20, p=base_params(fov0=-0.45 * np.pi, fov1=0.45 * np.pi,
                                                 rv=2666)),
        dict(name="mismatch_rv61", n=8, p=base_params(rv=61)),
        dict(name="dense_n60", n=60, p=base_params(width=120.0, height=120.0)),
    ]
    for sp in step_specs:
        p = sp["p"]
        n = sp["n"]
        st = swarm(rng, n, p["width"], p["height"], p["window_pad"], p["radius"],
                   sp.get("kappa"))
        radii = np.full(n, p["radius"])
        a0 = b0 = vv0 = None
        if sp.get("hetero"):
            radii = f32(rng.choice([5.0, 10.0, 15.0], n))
            a0 = f32(rng.uniform(0.1, 3, n)); b0 = f32(rng.uniform(0.1, 3, n))
            vv0 = f32(rng.uniform(0.5, 2, n))
            st["x"][1] = st["x"][0]; st["y"][1] = st["y"][0]        # coincident top-left
        if sp["name"] == "torus_n30":   # agents close across the seam
            st["x"][0] = f32(p["window_pad"] + 1.0); st["x"][1] = f32(p["window_pad"] +
                                                                     p["width"] - 25.0)
            st["y"][0] = st["y"][1]
        new, vpf, terms = ref_step(mods, p, st, radii, a0, b0, vv0)
        scs.append(dict(name=sp["name"], params=params_vec(p), radii=radii,
                        x=st["x"], y=st["y"], theta=st["theta"], v=st["v"],
                        alp0=np.zeros(0) if a0 is None else a0,
                        bet0=np.zeros(0) if b0 is None else b0,
                        v0=np.zeros(0) if vv0 is None else vv0,
                        x_new=new["x"], y_new=new["y"], theta_new=new["theta"],
                        v_new=new["v"], vpf=np.packbits(vpf, axis=1), terms=terms))
    np.savez_compressed(os.path.join(HERE, "steps.npz"),
                        **{f"c{i}_{k}": np.asarray(v) for i, c in enumerate(scs)
                           for k, v in c.items()}, count=len(scs))

    # ---------------------------------------------------------------- sequential steps
    qcs = []
    for (n, p) in ((6, base_params(rv=600)), (12, base_params(boundary=1, rv=400))):
        st = swarm(rng, n, p["width"], p["height"], p["window_pad"], p["radius"])
        radii = np.full(n, p["radius"])
        traj = [st]
        cur = st
        for _ in range(3):
            cur, _, _ = ref_step(mods, p, cur, radii, sequential=True)
            traj.append(cur)
        qcs.append(dict(params=params_vec(p), radii=radii,
                        traj=np.array([[t[k] for k in ("x", "y", "theta", "v")]
                                       for t in traj])))
    np.savez_compressed(os.path.join(HERE, "sequential.npz"),
                        **{f"c{i}_{k}": np.asarray(v) for i, c in enumerate(qcs)
                           for k, v in c.items()}, count=len(qcs))

    # ---------------------------------------------------------------- social channel
    class _Ag:
        pass

    ocs = []
    for case in range(24):
        n = int(rng.integers(3, 40))
        W = 400.0
        R = 10.0
        rv = int(rng.choice([64, 400, 1200]))
        x = f32(rng.uniform(30, 30 + W, n)); y = f32(rng.uniform(30, 30 + W, n))
        th = f32(rng.uniform(0, 2 * np.pi, n))
        exploit = (rng.random(n) < 0.5).astype(np.int32)
        patch = np.where(exploit > 0, rng.integers(-1, 3, n), -1).astype(np.int32)
        vr = float(rng.choice([80.0, 200.0, 1000.0]))
        vex = bool(case % 3 != 0)
        pw = bool(case % 2 == 0)
        fov = (-np.pi, np.pi) if case % 4 else (-0.6 * np.pi, 0.6 * np.pi)
        if case == 5:        # one occluder strictly inside a farther interval
            x[1] = f32(x[0] + 60); y[1] = y[0]; x[2] = f32(x[0] + 30); y[2] = y[0]
            exploit[1] = 1; patch[1] = 2; exploit[2] = 0
        ags = []
        for j in range(n):
            a = object.__new__(Agent)
            a.id = j
            a.position = np.array([x[j], y[j]], np.float64)
            a.radius = R
            a.orientation = float(th[j])
            a.v_field_res = rv
            a.FOV = fov
            a.vision_range = vr
            a.visual_exclusion = vex
            a.exclude_agents_same_patch = pw
            a.exploited_patch_id = int(patch[j])
            a._mode = "exploit" if exploit[j] else "explore"
            a.get_mode = (lambda s=a: s._mode)
            ags.append(a)
        fields = []
        for a in ags:
            a.calc_social_V_proj(ags)
            fields.append(np.asarray(a.soc_v_field) > 0)
        ocs.append(dict(rv=rv, x=x, y=y, theta=th, exploit=exploit, patch=patch, vr=vr,
                        vex=int(vex), pw=int(pw), fov=np.array(fov), R=R,
                        out=np.packbits(np.array(fields, np.uint8), axis=1)))
    np.savez_compressed(os.path.join(HERE, "social.npz"),
                        **{f"c{i}_{k}": np.asarray(v) for i, c in enumerate(ocs)
                           for k, v in c.items()}, count=len(ocs))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ABM_REFERENCE_ROOT")
    if not root:
        sys.exit(f"usage: python {os.path.basename(__file__)} REFERENCE_ROOT "
                 "(or set ABM_REFERENCE_ROOT): the root of the scioip34/ABM source tree")
    main(root)
