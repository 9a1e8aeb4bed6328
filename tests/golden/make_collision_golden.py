"""Generate tests/golden/collision.npz: foraging steps WITH agent-agent collisions, run by the
REFERENCE's own code.

Run from the repository root in a container that has the reference checkout:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_collision_golden.py /path/to/reference

Each case is one foraging step (make_forage_golden.reference_step) preceded by the
agent-agent block of Simulation.start (abm/simulation/sims.py:735-784) on crowded arenas:
the collision lists of pygame.sprite.groupcollide with the reference's
interactions.within_group_collision, the reference's own
Simulation.agent_agent_collision_proximity for every list (it computes each agent's
proximity field with Agent.projection_field), and the collided-agent bookkeeping of the loop.
pygame is not installed here: its groupcollide iteration (every sprite of the group in order,
with the list of group members it collides with) and collide_circle (circles of the sprites'
`radius` around their rect centres; a rect holds int(position) and the size of the agent's
2R x 2R image) are restated in this script.  After the block the GPU step stores orientation
and speed as float32, and so does the case here.
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


class _Rect:
    """pygame.Rect's integer geometry: x, y truncated, centre = x + w // 2."""

    def __init__(self, x, y, w, h):
        self.x, self.y, self.w, self.h = int(x), int(y), int(w), int(h)

    @property
    def centerx(self):
        return self.x + self.w // 2

    @property
    def centery(self):
        return self.y + self.h // 2


def _collide_circle(left, right):
    """pygame.sprite.collide_circle for sprites with a `radius` attribute."""
    dx = left.rect.centerx - right.rect.centerx
    dy = left.rect.centery - right.rect.centery
    return dx ** 2 + dy ** 2 <= (left.radius + right.radius) ** 2


def make_case(rng, case):
    from abm_gb300.foraging import ForageParams, initial_state
    W = float(rng.choice([200.0, 260.0]))
    p = ForageParams(pooling_time=0, teleport_exploit=bool(case % 3 != 1),
                     Tau=int(rng.choice([5, 10])), regenerate_patches=False,
                     rv=int(rng.choice([120, 121, 400, 1200])),
                     vision_range=float(rng.choice([30.0, 150.0, 2000.0])),
                     visual_exclusion=bool(case % 4 != 3), patchwise_exclusion=bool(case % 2),
                     width=W, height=W, consumption=1.0, min_resc_quality=0.5,
                     max_resc_quality=1.5, collide_agents=True,
                     ghost_mode=bool(case % 5 not in (1, 3)))
    n = int(rng.integers(10, 28))
    ag, pt = initial_state(p, n, 3, seed=int(rng.integers(1 << 30)))
    pt["quality"][:] = rng.uniform(0.5, 1.5, 3)
    pt["left"][:] = np.where(rng.random(3) < 0.3, rng.uniform(0.2, 3.0, 3), 300.0)
    lo, hi = p.window_pad - p.agent_radius + 1, p.window_pad + W - p.agent_radius - 1
    x = rng.uniform(lo, hi, n)
    y = rng.uniform(lo, hi, n)
    # clusters: agents placed 5-30 px from an earlier one (several lists per agent), a few
    # exactly on top of another one (coincident agents are skipped by the projection)
    for i in range(1, n):
        u = rng.random()
        if u < 0.45:
            j = int(rng.integers(0, i))
            r, a = rng.uniform(5, 30), rng.uniform(0, 2 * np.pi)
            x[i] = np.clip(x[j] + r * np.cos(a), lo, hi)
            y[i] = np.clip(y[j] + r * np.sin(a), lo, hi)
        elif u < 0.52:
            j = int(rng.integers(0, i))
            x[i], y[i] = x[j], y[j]
    ag["x"][:], ag["y"][:] = x, y
    ag["theta"][:] = rng.uniform(0, 2 * np.pi, n)
    ag["v"][:] = rng.choice([0.0, 0.5, 1.0], n)
    ag["w"][:] = rng.uniform(-1, 1, n)
    ag["u"][:] = rng.uniform(-1, 1, n)
    ag["collected_before"][:] = rng.integers(0, 20, n)
    ag["collected"][:] = ag["collected_before"] + rng.choice([0.0, 1.0], n)
    kind = rng.random(n)
    expl, coll = kind < 0.3, (kind >= 0.3) & (kind < 0.55)
    ag["override_mode"][:] = np.where(expl, 2, np.where(coll, 4, -1))
    ag["mode"][:] = np.where(expl, 2, np.where(coll, 4, rng.integers(0, 2, n)))
    ag["env_status"][:] = rng.integers(-1, 2, n)
    ag["env_status_before"][:] = rng.integers(-1, 2, n)
    ag["pool_success"][:] = rng.integers(0, 2, n)
    ag["patch_id"][:] = np.where(expl, rng.integers(-1, 4, n), -1)
    ag["novelty"][:] = rng.integers(0, 1 << p.Tau, n)
    uniforms = rng.random(n)
    for k in ("x", "y", "theta", "v"):
        ag[k] = np.asarray(ag[k], np.float32)
    return p, ag, pt, uniforms


def collision_block(p, agents, sims, itra):
    """sims.py:735-784 with the reference's own collision functions."""
    for a in agents:                      # Agent.draw_update: rect.x = position[0], ...
        a.rect = _Rect(a.position[0], a.position[1], 2 * a.radius, 2 * a.radius)
    sim = types.SimpleNamespace(agents=agents, ghost_mode=p.ghost_mode,
                                teleport_exploit=p.teleport_exploit)
    proximity_distance = 2
    for agent in agents:
        agent.radius += proximity_distance
    group = {}                            # pygame.sprite.groupcollide(agents, agents, ...)
    for a1 in agents:
        hits = [a2 for a2 in agents if itra.within_group_collision(a1, a2)]
        if hits:
            group[a1] = hits
    for agent in agents:
        agent.radius -= proximity_distance
    collided = []
    for agent1, agent2 in group.items():
        sims.Simulation.agent_agent_collision_proximity(sim, agent1, agent2)
        for b in agent2:
            if sim.teleport_exploit:
                if agent1.get_mode() != "exploit":
                    collided.append(agent1)
                if b.get_mode() != "exploit":
                    collided.append(b)
            else:
                if not sim.ghost_mode:
                    collided.append(agent1)
                    collided.append(b)
                elif agent1.get_mode() != "exploit" and b.get_mode() != "exploit":
                    collided.append(agent1)
                    collided.append(b)
    for agent in agents:
        if agent not in collided and agent.get_mode() == "collide":
            agent.set_mode("explore")
        if agent in collided and agent.get_mode() == "collide":
            sims.notify_agent(agent, -1)
    for a in agents:                      # stored as float32 by the GPU step
        a.orientation = float(np.float32(a.orientation))
        a.velocity = float(np.float32(a.velocity))
    return sum(len(v) for v in group.values())


def main(ref_root):
    import make_forage_golden as mfg
    mfg.install_foraging_shims(ref_root)
    sys.modules["pygame"].sprite.collide_circle = _collide_circle
    from abm.agent import supcalc
    from abm.agent.agent import Agent
    from abm.environment.rescource import Rescource
    from abm.simulation import interactions as itra
    from abm.simulation import sims
    rng = np.random.default_rng(20261205)
    cases, total = [], 0
    for case in range(20):
        p, ag, pt, uni = make_case(rng, case)
        pairs = []
        out, pout, soc = mfg.reference_step(
            p, ag, pt, uni, Agent, Rescource, sims, supcalc,
            before_interaction=lambda agents: pairs.append(collision_block(p, agents, sims,
                                                                            itra)))
        total += pairs[0]
        fp, ip, seed = p.oracle_arrays()
        c = {"fp": fp, "ip": ip, "uniforms": uni, "soc": np.packbits(soc, axis=1),
             "pairs": pairs[0]}
        c.update({"in_" + k: v for k, v in ag.items()})
        c.update({"pin_" + k: v for k, v in pt.items()})
        c.update({"out_" + k: v for k, v in out.items()})
        c.update({"pout_" + k: v for k, v in pout.items()})
        cases.append(c)
    np.savez_compressed(os.path.join(HERE, "collision.npz"),
                        **{f"c{i}_{k}": np.asarray(v) for i, c in enumerate(cases)
                           for k, v in c.items()}, count=len(cases))
    print(f"collision.npz written to {HERE} ({total} collision list entries)")


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ABM_REFERENCE_ROOT")
    if not root:
        sys.exit(f"usage: python {os.path.basename(__file__)} REFERENCE_ROOT "
                 "(or set ABM_REFERENCE_ROOT): the root of the scioip34/ABM source tree")
    main(root)
