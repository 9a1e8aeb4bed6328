"""Generate tests/golden/recording.json with the REFERENCE's RAM recorder.

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_recording_golden.py /path/to/reference

Synthetic agents and patches (values exactly representable in the GPU recording: float32
positions / orientations / speeds) go through the reference's own ifdb.save_agent_data_RAM and
ifdb.save_resource_data_RAM (abm/monitoring/ifdb.py:55-96, :223-260) for a few steps, one patch
being moved and refilled half-way like a regeneration; the JSON the reference writes from them
(json.dump of its dictionaries, ifdb.py:412-434) is stored next to the same states in the
layout of abm_gb300.foraging.ForagingSim.recording().
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

MODES = ["explore", "exploit", "relocate", "collide"]


def main(ref_root):
    import make_forage_golden
    make_forage_golden.install_foraging_shims(ref_root)
    from abm.monitoring import ifdb
    rng = np.random.default_rng(77)
    n, n_p, steps, rv = 4, 2, 5, 96
    words = (rv + 31) // 32

    class Obj:
        pass

    agents = [Obj() for _ in range(n)]
    patches = [Obj() for _ in range(n_p)]
    for i, a in enumerate(agents):
        a.id = i
    for k, r in enumerate(patches):
        r.id = k + 1
        r.radius = 30.0
    rec = {key: np.zeros((n, steps)) for key in ("posx", "posy", "orientation", "velocity", "w",
                                                  "u", "ipriv", "collected", "mode",
                                                  "patch_id")}
    rec.update({key: np.zeros((n_p, steps)) for key in ("res_posx", "res_posy", "res_left",
                                                          "res_quality", "res_id")})
    soc = np.zeros((n, steps, words), np.uint32)
    ifdb.agents_dict = {}
    ifdb.resources_dict = {}
    for t in range(steps):
        for i, a in enumerate(agents):
            a.position = np.array([np.float32(rng.uniform(-5, 900)),
                                   np.float32(rng.uniform(-5, 900))], np.float64)
            a.orientation = float(np.float32(rng.uniform(0, 2 * np.pi)))
            a.velocity = float(np.float32(rng.uniform(-1, 2)))
            a.w, a.u = float(rng.uniform(-1, 1)), float(rng.uniform(-1, 1))
            a.I_priv = float(rng.choice([0.0, 1.0, 2.0, 3.5]))
            m = int(rng.integers(0, 4))
            a.mode = MODES[m]
            a.collected_r = float(rng.integers(0, 50))
            a.exploited_patch_id = int(rng.integers(-1, 3))
            V = (rng.random(rv) < 0.3).astype(np.float64)
            V[: int(rng.integers(0, 5))] = 1.0
            a.soc_v_field = V
            for key, val in (("posx", int(a.position[0])), ("posy", int(a.position[1])),
                             ("orientation", a.orientation), ("velocity", a.velocity),
                             ("w", a.w), ("u", a.u), ("ipriv", a.I_priv), ("mode", m),
                             ("collected", a.collected_r),
                             ("patch_id", a.exploited_patch_id)):
                rec[key][i, t] = val
            bits = np.packbits(V.astype(np.uint8), bitorder="little")
            padded = np.zeros(words * 4, np.uint8)
            padded[: len(bits)] = bits
            soc[i, t] = padded.view("<u4")
        for k, r in enumerate(patches):
            if t == 0 or (k == 1 and t == 3):     # slot 1 regenerated at step 3
                r.position = np.array([float(rng.integers(30, 900)), float(rng.integers(30, 900))])
                r.resc_left = 100.0
            r.resc_left = float(r.resc_left - rng.choice([0.0, 0.5, 1.0]))
            r.unit_per_timestep = float(rng.uniform(0.1, 1.0))
            for key, val in (("res_posx", int(r.position[0])), ("res_posy", int(r.position[1])),
                             ("res_left", r.resc_left), ("res_quality", r.unit_per_timestep),
                             ("res_id", r.id)):
                rec[key][k, t] = val
        ifdb.save_agent_data_RAM(agents, t + 1)
        ifdb.save_resource_data_RAM(patches, t + 1)
    out = {"rv": rv, "n": n, "n_patches": n_p, "steps": steps,
           "rec": {k: v.tolist() for k, v in rec.items()},
           "soc_bits": soc.astype(np.int64).tolist(), "radius": [30.0] * n_p,
           "agent_json": json.dumps(ifdb.agents_dict),
           "resource_json": json.dumps(ifdb.resources_dict)}
    with open(os.path.join(HERE, "recording.json"), "w") as f:
        json.dump(out, f)
    print("recording.json written to", HERE)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ABM_REFERENCE_ROOT")
    if not root:
        sys.exit(f"usage: python {os.path.basename(__file__)} REFERENCE_ROOT "
                 "(or set ABM_REFERENCE_ROOT): the root of the scioip34/ABM source tree")
    main(root)
