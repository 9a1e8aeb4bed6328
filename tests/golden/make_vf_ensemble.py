"""Generate tests/golden/vf_ensemble.npz: polarisation series of whole REFERENCE flocking runs.

Run from the repository root in a container that has the reference checkout:

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_vf_ensemble.py /path/to/reference

Each run is the plain visual-flocking workload of N=10 agents (radius 10, 500 x 500 walls,
Rv=1200 over a field of view of 2 pi, V0=1, ALP0=BET0=1, ALP1=BET1=0.08, speeds starting at 0)
played by the reference's own VFAgent methods in its own order: every step each agent, in
group order, computes its field from the agents as they are at that moment (those before it
already moved, VFSimulation.step_sim, vf_sims.py:291-302), acts, moves and reflects from the
walls (vf_agent.py:52-77).  Positions and headings start uniform from numpy's generator seeded
per run (float32 values, the precision of the GPU state).  Saved per run: the initial state and
the polarisation |sum_i (cos theta_i, sin theta_i)| / N after every step
(data_loader.py:1818-1824).  vf_ensemble.npz holds the walls arena, vf_ensemble_torus.npz the
same runs on the torus (VFAgent.teleport_infinite_arena, vf_agent.py:188-204).
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

N, T, RUNS = 10, 1000, 32


def initial(seed, p):
    rng = np.random.default_rng(seed)
    pad, R, W, H = p["window_pad"], p["radius"], p["width"], p["height"]
    f32 = lambda a: np.asarray(a, np.float32).astype(np.float64)
    return {"x": f32(rng.uniform(pad - R, pad + W - R, N)),
            "y": f32(rng.uniform(pad - R, pad + H - R, N)),
            "theta": f32(rng.uniform(0, 2 * np.pi, N)), "v": np.zeros(N)}


def play(mods, p, name):
    import make_golden
    seeds = np.arange(RUNS) + 500
    init = {k: np.zeros((RUNS, N)) for k in ("x", "y", "theta")}
    pol = np.zeros((RUNS, T))
    radii = np.full(N, p["radius"])
    t0 = time.time()
    for r, seed in enumerate(seeds):
        st = initial(int(seed), p)
        for k in init:
            init[k][r] = st[k]
        for t in range(T):
            st, _, _ = make_golden.ref_step(mods, p, st, radii, sequential=True)
            pol[r, t] = np.hypot(np.cos(st["theta"]).sum(), np.sin(st["theta"]).sum()) / N
        print(f"{name} run {r}: final polarisation {pol[r, -1]:.4f} ({time.time() - t0:.0f} s)")
    np.savez_compressed(os.path.join(HERE, name), seeds=seeds, pol=pol,
                        params=make_golden.params_vec(p), **{f"init_{k}": v for k, v in init.items()})
    print(name, "written to", HERE)


def main(ref_root):
    import make_golden
    make_golden.install_shims(ref_root)
    from abm.projects.visual_flocking.vf_agent.vf_agent import VFAgent
    from abm.projects.visual_flocking.vf_contrib import vf_params
    mods = (VFAgent, vf_params)
    play(mods, make_golden.base_params(), "vf_ensemble.npz")                      # walls
    play(mods, make_golden.base_params(boundary=1), "vf_ensemble_torus.npz")      # torus


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ABM_REFERENCE_ROOT")
    if not root:
        sys.exit(f"usage: python {os.path.basename(__file__)} REFERENCE_ROOT "
                 "(or set ABM_REFERENCE_ROOT): the root of the scioip34/ABM source tree")
    main(root)
