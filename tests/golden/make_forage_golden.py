"""Generate tests/golden/forage.npz by running the REFERENCE foraging step.

Run from the repository root in a container that has the reference checkout:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_forage_golden.py /path/to/reference

One step of the reference's foraging simulation (abm/simulation/sims.py:789-858 without
agent-agent collisions, then Agent.update, abm/agent/agent.py:213-283) from seeded states
chosen to reach every branch: agents inside patches and outside, exploiting and not, pooling
flags, w / u on both sides of the thresholds, patches with a few units left so that one agent
empties them, teleporting on and off, several pooling times and Tau.  The resource phase calls
the reference's own notify_agent, Simulation.bias_agent_towards_res_center and
Rescource.deplete in the order of the sims.py loop; the update calls Agent.update on copies of
the post-interaction snapshot (one copy per focal agent, so every agent sees the same
snapshot, as the GPU step does), with np.random.uniform returning the case's injected draw
(the random walk's only random number, supcalc.py:38-47).  Patch regeneration is off here
(the reference draws new patches from numpy's global generator).  Besides make_golden.py's
shims, pygame drawing, influxdb and matplotlib are stubbed; Agent.draw_update (drawing only)
is replaced by a no-op.  The reference is never modified.
"""
from __future__ import annotations

import copy
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

MODE_ID = {"explore": 0, "relocate": 1, "exploit": 2, "pool": 3, "collide": 4}


def install_foraging_shims(ref_root):
    import make_golden
    make_golden.install_shims(ref_root)
    pg = sys.modules["pygame"]

    class _Any:
        def __init__(self, *a, **k):
            pass

        def __getattr__(self, k):
            return _Any()

        def __call__(self, *a, **k):
            return _Any()

    for name in ("draw", "gfxdraw", "mask", "font", "display", "time", "event"):
        setattr(pg, name, _Any())
    pg.Surface = _Any
    pg.sprite.Group = _Any
    sys.modules["pygame.gfxdraw"] = pg.gfxdraw
    inf = types.ModuleType("influxdb")
    inf.InfluxDBClient = _Any
    inf.DataFrameClient = _Any
    sys.modules["influxdb"] = inf


def f32(a):
    return np.asarray(a, dtype=np.float32)


def make_case(rng, case):
    from abm_gb300.foraging import ForageParams, initial_state
    p = ForageParams(pooling_time=int(rng.choice([0, 0, 2])),
                     teleport_exploit=bool(case % 3 != 1), Tau=int(rng.choice([1, 5, 10, 32])),
                     regenerate_patches=False, rv=int(rng.choice([120, 400, 1200])),
                     vision_range=float(rng.choice([150.0, 400.0, 2000.0])),
                     visual_exclusion=bool(case % 4 != 3), patchwise_exclusion=bool(case % 2),
                     width=500.0, height=500.0, consumption=float(rng.choice([1.0, 2.0])),
                     min_resc_quality=0.5, max_resc_quality=1.5)
    n = int(rng.integers(8, 40))
    ag, pt = initial_state(p, n, 3, seed=int(rng.integers(1 << 30)))
    pt["quality"][:] = rng.uniform(0.5, 1.5, 3)
    pt["left"][:] = np.where(rng.random(3) < 0.5, rng.uniform(0.2, 3.0, 3), 300.0)
    # put about a third of the agents inside patches, at random offsets from the centre
    inside = rng.random(n) < 0.35
    for i in np.where(inside)[0]:
        k = int(rng.integers(0, 3))
        r = rng.uniform(0, 0.9 * pt["radius"][k])
        a = rng.uniform(0, 2 * np.pi)
        ag["x"][i] = pt["x"][k] + pt["radius"][k] + r * np.cos(a) - p.agent_radius
        ag["y"][i] = pt["y"][k] + pt["radius"][k] + r * np.sin(a) - p.agent_radius
    ag["theta"][:] = rng.uniform(0, 2 * np.pi, n)
    ag["v"][:] = rng.choice([0.0, 0.5, 1.0, 1.7], n)
    ag["w"][:] = rng.uniform(-1, 1, n)
    ag["u"][:] = rng.uniform(-1, 1, n)
    ag["collected_before"][:] = rng.integers(0, 20, n)
    ag["collected"][:] = ag["collected_before"] + rng.choice([0.0, 0.0, 1.0, 0.5], n)
    expl = rng.random(n) < 0.4
    ag["override_mode"][:] = np.where(expl, 2, -1)
    ag["mode"][:] = np.where(expl, 2, rng.integers(0, 2, n))
    ag["env_status"][:] = rng.integers(-1, 2, n)
    ag["env_status_before"][:] = rng.integers(-1, 2, n)
    ag["pool_success"][:] = rng.integers(0, 2, n)
    ag["patch_id"][:] = np.where(expl, rng.integers(-1, 4, n), -1)
    ag["novelty"][:] = rng.integers(0, 1 << min(p.Tau, 31), n) & rng.integers(0, 2, n) * -1
    uniforms = rng.random(n)
    for k in ("x", "y", "theta", "v"):
        ag[k] = f32(ag[k])
    return p, ag, pt, uniforms


def reference_step(p, ag, pt, uniforms, Agent, Rescource, sims, supcalc,
                   before_interaction=None):
    """The reference step for one case; returns (agents dict, patches dict, soc fields).
    before_interaction(agents), when given, runs on the reference agents before the
    agent-resource interaction (the agent-agent collision block of sims.py:735-784)."""
    from abm.contrib import movement_params
    movement_params.exp_theta_min, movement_params.exp_theta_max = (p.exp_theta_min,
                                                                    p.exp_theta_max)
    movement_params.reloc_theta_max = p.reloc_theta_max
    n = len(ag["x"])
    agents = []
    for i in range(n):
        a = object.__new__(Agent)
        a.id = i
        a.radius = p.agent_radius
        a.position = np.array([float(ag["x"][i]), float(ag["y"][i])], np.float64)
        a.orientation = float(ag["theta"][i])
        a.velocity = float(ag["v"][i])
        a.v_field_res = p.rv
        a.FOV = (-p.fov * np.pi, p.fov * np.pi)
        a.vision_range = p.vision_range
        a.visual_exclusion = p.visual_exclusion
        a.exclude_agents_same_patch = p.patchwise_exclusion
        a.pooling_time = p.pooling_time
        a.consumption = p.consumption
        a.collected_r = float(ag["collected"][i])
        a.collected_r_before = float(ag["collected_before"][i])
        a.exploited_patch_id = int(ag["patch_id"][i])
        inv = {v: k for k, v in MODE_ID.items()}
        a.mode = inv[int(ag["mode"][i])]
        a.overriding_mode = None if ag["override_mode"][i] < 0 else inv[int(ag["override_mode"][i])]
        a.soc_v_field = np.zeros(p.rv)
        a.vis_field_source_data = {}
        a.is_moved_with_cursor = 0
        a.S_wu, a.T_w, a.w = p.S_wu, p.T_w, float(ag["w"][i])
        a.Eps_w, a.g_w, a.B_w, a.w_max = p.Eps_w, p.g_w, p.B_w, p.w_max
        a.I_priv = 0
        a.novelty = np.array([(int(ag["novelty"][i]) >> k) & 1 for k in range(p.Tau)], float)
        a.S_uw, a.T_u, a.u = p.S_uw, p.T_u, float(ag["u"][i])
        a.Eps_u, a.g_u, a.B_u, a.u_max = p.Eps_u, p.g_u, p.B_u, p.u_max
        a.F_N, a.F_R = p.F_N, p.F_R
        a.max_exp_vel, a.exp_stop_ratio = p.exp_vel_max, p.exp_stop_ratio
        a.env_status = int(ag["env_status"][i])
        a.env_status_before = int(ag["env_status_before"][i])
        a.pool_success = int(ag["pool_success"][i])
        a.WIDTH, a.HEIGHT, a.window_pad = p.width, p.height, p.window_pad
        a.boundaries_x = [p.window_pad, p.window_pad + p.width]
        a.boundaries_y = [p.window_pad, p.window_pad + p.height]
        a.draw_update = lambda: None
        agents.append(a)
    rescs = []
    for k in range(len(pt["x"])):
        r = object.__new__(Rescource)
        r.id = int(pt["id"][k])
        r.radius = float(pt["radius"][k])
        r.position = np.array([pt["x"][k], pt["y"][k]], np.float64)
        r.center = (r.position[0] + r.radius, r.position[1] + r.radius)
        r.resc_units = float(pt["units"][k])
        r.resc_left = float(pt["left"][k])
        r.unit_per_timestep = float(pt["quality"][k])
        rescs.append(r)
    if before_interaction is not None:
        before_interaction(agents)
    # ---- agent-resource interaction, sims.py:789-855 (refine_ar_overlap_group, sims.py:45-56,
    #      selects the agents whose centre is inside a patch; pygame's circle test before it
    #      accepts a superset of them)
    group = {r: [a for a in agents if supcalc.distance(r, a) < r.radius] for r in rescs}
    on = []
    for resc, ags in group.items():
        destroy_resc = 0
        for agent in ags:
            sims.Simulation.bias_agent_towards_res_center(None, agent, resc)
            if destroy_resc:
                sims.notify_agent(agent, -1)
            else:
                if (agent.get_mode() in ["pool", "relocate"] and agent.pool_success) \
                        or agent.pooling_time == 0:
                    sims.notify_agent(agent, 1, resc.id)
                    if p.teleport_exploit:
                        agent.position = resc.position + resc.radius - agent.radius
                if agent.get_mode() == "exploit":
                    depl_units, destroy_resc = resc.deplete(agent.consumption)
                    agent.collected_r_before = agent.collected_r
                    agent.collected_r += depl_units
                    if destroy_resc:
                        for b in ags:
                            sims.notify_agent(b, -1)
            on.append(agent)
        if destroy_resc:
            resc.id = -1          # kill_resource without regeneration
    for agent in agents:
        if agent not in on:
            if (agent.get_mode() in ["pool", "relocate"] and agent.pool_success) \
                    or agent.pooling_time == 0:
                sims.notify_agent(agent, -1)
            elif agent.get_mode() == "exploit":
                sims.notify_agent(agent, -1)
    # the GPU step stores positions and orientation as float32 between the two phases
    for a in agents:
        a.position = np.array([float(np.float32(a.position[0])),
                               float(np.float32(a.position[1]))], np.float64)
        a.orientation = float(np.float32(a.orientation))
    # ---- agent update from the snapshot (one copy per focal agent)
    snap = copy.deepcopy(agents)
    out = {k: np.zeros(n, np.float64) for k in ("x", "y", "theta", "v", "w", "u", "collected",
                                                  "collected_before")}
    for k in ("mode", "override_mode", "env_status", "env_status_before", "pool_success",
              "patch_id", "novelty"):
        out[k] = np.zeros(n, np.int64)
    soc = np.zeros((n, p.rv), np.uint8)
    real_uniform = np.random.uniform
    for i in range(n):
        world = copy.deepcopy(snap)
        for a in world:
            a.draw_update = lambda: None
        np.random.uniform = lambda lo, hi, _u=float(uniforms[i]): lo + (hi - lo) * _u
        try:
            world[i].update(world)
        finally:
            np.random.uniform = real_uniform
        a = world[i]
        soc[i] = (np.asarray(a.soc_v_field) > 0).astype(np.uint8)
        out["x"][i], out["y"][i] = a.position
        out["theta"][i], out["v"][i] = a.orientation, a.velocity
        out["w"][i], out["u"][i] = a.w, a.u
        out["collected"][i], out["collected_before"][i] = a.collected_r, a.collected_r_before
        out["mode"][i] = MODE_ID[a.mode]
        out["override_mode"][i] = -1 if a.overriding_mode is None else MODE_ID[a.overriding_mode]
        out["env_status"][i], out["env_status_before"][i] = a.env_status, a.env_status_before
        out["pool_success"][i], out["patch_id"][i] = a.pool_success, a.exploited_patch_id
        out["novelty"][i] = sum(int(v) << k for k, v in enumerate(a.novelty))
    pout = {"left": np.array([r.resc_left for r in rescs]), "id": np.array([r.id for r in rescs])}
    return out, pout, soc


def main(ref_root):
    install_foraging_shims(ref_root)
    from abm.agent import supcalc
    from abm.agent.agent import Agent
    from abm.environment.rescource import Rescource
    from abm.simulation import sims
    rng = np.random.default_rng(20261204)
    cases = []
    for case in range(16):
        p, ag, pt, uni = make_case(rng, case)
        out, pout, soc = reference_step(p, ag, pt, uni, Agent, Rescource, sims, supcalc)
        fp, ip, seed = p.oracle_arrays()
        c = {"fp": fp, "ip": ip, "uniforms": uni, "soc": np.packbits(soc, axis=1)}
        c.update({"in_" + k: v for k, v in ag.items()})
        c.update({"pin_" + k: v for k, v in pt.items()})
        c.update({"out_" + k: v for k, v in out.items()})
        c.update({"pout_" + k: v for k, v in pout.items()})
        cases.append(c)
    np.savez_compressed(os.path.join(HERE, "forage.npz"),
                        **{f"c{i}_{k}": np.asarray(v) for i, c in enumerate(cases)
                           for k, v in c.items()}, count=len(cases))
    print("forage.npz written to", HERE)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ABM_REFERENCE_ROOT")
    if not root:
        sys.exit(f"usage: python {os.path.basename(__file__)} REFERENCE_ROOT "
                 "(or set ABM_REFERENCE_ROOT): the root of the scioip34/ABM source tree")
    main(root)
