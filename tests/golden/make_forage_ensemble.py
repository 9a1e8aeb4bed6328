"""Generate tests/golden/forage_ensemble.npz: foraging efficiency of whole REFERENCE runs.

Run from the repository root in a container that has the reference checkout:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_forage_ensemble.py /path/to/reference

Each run plays the reference's foraging loop (abm/simulation/sims.py:789-858 without
agent-agent collisions, then Agent.update for every agent in group order, each seeing the
agents already updated this step — the reference's own sequential order) for T steps with the
reference's own functions (notify_agent, bias_agent_towards_res_center, Rescource.deplete,
Agent.update) and numpy's global generator seeded per run for the random walk and for patch
regeneration (add_new_resource_patch's rules, sims.py:332-374).  The initial agents and patches
are abm_gb300.foraging.initial_state(seed), the placement the GPU runs start from.  Saved per
run: the per-agent foraging efficiency over [T0, T) (data_loader.py:1333-1346).
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

N_AGENTS, N_PATCHES, T, T0, RUNS = 30, 3, 1500, 500, 12


def ensemble_params():
    from abm_gb300.foraging import ForageParams
    return ForageParams(width=500.0, height=500.0, agent_radius=10.0, patch_radius=30.0,
                        min_resc_units=150, max_resc_units=250, min_resc_quality=1.0,
                        max_resc_quality=1.0, consumption=1.0, rv=400, fov=0.5,
                        vision_range=300.0, visual_exclusion=True, teleport_exploit=False,
                        pooling_time=0)


def run_reference(seed, Agent, Rescource, sims, supcalc):
    from abm_gb300.foraging import initial_state
    from make_forage_golden import MODE_ID
    import make_forage_golden as mfg
    p = ensemble_params()
    ag, pt = initial_state(p, N_AGENTS, N_PATCHES, seed=seed)
    # reference objects (the same construction as the per-step fixtures)
    agents, rescs = build_objects(p, ag, pt, Agent, Rescource)
    np.random.seed(seed)
    from abm.contrib import movement_params
    movement_params.exp_theta_min, movement_params.exp_theta_max = (p.exp_theta_min,
                                                                    p.exp_theta_max)
    movement_params.reloc_theta_max = p.reloc_theta_max
    c0 = None
    for t in range(T):
        if t == T0:
            c0 = np.array([a.collected_r for a in agents])
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
                    if agent.get_mode() == "exploit":
                        depl_units, destroy_resc = resc.deplete(agent.consumption)
                        agent.collected_r_before = agent.collected_r
                        agent.collected_r += depl_units
                        if destroy_resc:
                            for b in ags:
                                sims.notify_agent(b, -1)
                on.append(agent)
            if destroy_resc:
                regenerate(p, resc, rescs)
        for agent in agents:
            if agent not in on:
                if (agent.get_mode() in ["pool", "relocate"] and agent.pool_success) \
                        or agent.pooling_time == 0:
                    sims.notify_agent(agent, -1)
                elif agent.get_mode() == "exploit":
                    sims.notify_agent(agent, -1)
        for agent in agents:            # pygame group order: each sees the updated ones
            agent.update(agents)
    c1 = np.array([a.collected_r for a in agents])
    return (c1 - c0) / (T - T0)


def regenerate(p, resc, rescs):
    """kill_resource + add_new_resource_patch(force_id) (sims.py:321-374) with numpy's global
    generator: integer position without patch overlap, units randint, quality uniform."""
    r = p.patch_radius
    others = [o for o in rescs if o is not resc]
    while True:
        x = np.random.randint(p.window_pad, p.width + p.window_pad - 2 * r)
        y = np.random.randint(p.window_pad, p.height + p.window_pad - 2 * r)
        units = np.random.randint(p.min_resc_units, p.max_resc_units)
        quality = np.random.uniform(p.min_resc_quality, p.max_resc_quality)
        cx, cy = x + r, y + r
        if all((cx - o.center[0]) ** 2 + (cy - o.center[1]) ** 2 >= (r + o.radius) ** 2
               for o in others):
            break
    resc.position = np.array([x, y], np.float64)
    resc.radius = r
    resc.center = (x + r, y + r)
    resc.resc_units = units
    resc.resc_left = units
    resc.unit_per_timestep = quality


def build_objects(p, ag, pt, Agent, Rescource):
    import make_forage_golden as mfg
    inv = {v: k for k, v in mfg.MODE_ID.items()}
    agents = []
    for i in range(len(ag["x"])):
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
        a.collected_r = 0.0
        a.collected_r_before = 0.0
        a.exploited_patch_id = -1
        a.mode = "explore"
        a.overriding_mode = None
        a.soc_v_field = np.zeros(p.rv)
        a.vis_field_source_data = {}
        a.is_moved_with_cursor = 0
        a.S_wu, a.T_w, a.w = p.S_wu, p.T_w, 0.0
        a.Eps_w, a.g_w, a.B_w, a.w_max = p.Eps_w, p.g_w, p.B_w, p.w_max
        a.I_priv = 0
        a.novelty = np.zeros(p.Tau)
        a.S_uw, a.T_u, a.u = p.S_uw, p.T_u, 0.0
        a.Eps_u, a.g_u, a.B_u, a.u_max = p.Eps_u, p.g_u, p.B_u, p.u_max
        a.F_N, a.F_R = p.F_N, p.F_R
        a.max_exp_vel, a.exp_stop_ratio = p.exp_vel_max, p.exp_stop_ratio
        a.env_status = 0
        a.env_status_before = 0
        a.pool_success = 0
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
    return agents, rescs


def main(ref_root):
    import make_forage_golden as mfg
    mfg.install_foraging_shims(ref_root)
    from abm.agent import supcalc
    from abm.agent.agent import Agent
    from abm.environment.rescource import Rescource
    from abm.simulation import sims
    effs = []
    for run in range(RUNS):
        effs.append(run_reference(1000 + run, Agent, Rescource, sims, supcalc))
        print(f"run {run}: mean efficiency {effs[-1].mean():.4f}", flush=True)
    p = ensemble_params()
    fp, ip, _ = p.oracle_arrays()
    np.savez_compressed(os.path.join(HERE, "forage_ensemble.npz"), eff=np.array(effs), fp=fp,
                        ip=ip, n_agents=N_AGENTS, n_patches=N_PATCHES, T=T, T0=T0,
                        seeds=1000 + np.arange(RUNS))
    print("forage_ensemble.npz written to", HERE)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ABM_REFERENCE_ROOT")
    if not root:
        sys.exit(f"usage: python {os.path.basename(__file__)} REFERENCE_ROOT "
                 "(or set ABM_REFERENCE_ROOT): the root of the scioip34/ABM source tree")
    main(root)
