"""Generate tests/golden/recording_zarr.json with the REFERENCE's own end-of-run writer.

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_zarr_golden.py /path/to/reference

Synthetic per-step states of foraging agents and patches, and of visual-flocking agents (whose
w, u, I_priv, mode, collected_r and exploited_patch_id keep the values Agent.__init__ gives
them, abm/agent/agent.py:68-126), go through the reference's RAM recorder
(ifdb.save_agent_data_RAM / save_resource_data_RAM, abm/monitoring/ifdb.py:55-96, :223-260) and
then through ifdb.save_ifdb_as_csv(use_ram=True, as_zar=True, save_extracted_vfield=True)
(ifdb.py:435-536).  The zarr package is absent here, so a stand-in module records what that
function asks of it: for every zarr.open its file name, shape, chunks and dtype, and the array
after all of the function's slice assignments (numpy assignment, as zarr's basic selection
does).  The fixture holds the inputs, the reference's agent JSON and those arrays.  Fields
include runs that wrap around pixel 0 and a full field, whose reconstruction by
reconstruct_VPF (abm/loader/helper.py:39-52) differs from the field.
"""
import json
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

MODES = ["explore", "exploit", "relocate", "collide"]


class _StubArray:
    def __init__(self, shape, chunks, dtype):
        self.data = np.zeros(shape, dtype=np.dtype(dtype))
        self.chunks = list(chunks)

    def __setitem__(self, key, value):
        self.data[key] = value


def _stub_zarr(store):
    mod = types.ModuleType("zarr")

    def _open(path, mode="r", shape=None, chunks=None, dtype=None, **kw):
        arr = _StubArray(shape, chunks, dtype)
        store[os.path.basename(path)] = arr
        return arr

    mod.open = _open
    return mod


def _fields(rng, n, rv):
    out = []
    for i in range(n):
        V = (rng.random(rv) < 0.3).astype(np.float64)
        kind = i % 5
        if kind == 0:
            V[: int(rng.integers(1, 5))] = 1.0       # a run from pixel 0 ...
            V[-int(rng.integers(1, 4)):] = 1.0       # ... that wraps around
        elif kind == 1:
            V[:] = 0.0
        elif kind == 2:
            V[:] = 1.0
        out.append(V)
    return out


def _run(ifdb, agents, patches, steps, rv, rng, forage):
    ifdb.agents_dict = {}
    ifdb.resources_dict = {}
    n, n_p = len(agents), len(patches)
    rec = {k: np.zeros((n, steps)) for k in ("posx", "posy", "orientation", "velocity", "w",
                                              "u", "ipriv", "collected", "mode", "patch_id")}
    rec.update({k: np.zeros((n_p, steps)) for k in ("res_posx", "res_posy", "res_left",
                                                     "res_quality", "res_id")})
    words = (rv + 31) // 32
    soc = np.zeros((n, steps, words), np.uint32)
    for t in range(steps):
        fields = _fields(rng, n, rv)
        for i, a in enumerate(agents):
            a.position = np.array([np.float32(rng.uniform(-5, 900)),
                                   np.float32(rng.uniform(-5, 900))], np.float64)
            a.orientation = float(np.float32(rng.uniform(0, 2 * np.pi)))
            a.velocity = float(np.float32(rng.uniform(-1, 2)))
            if forage:
                a.w, a.u = float(rng.uniform(-1, 1)), float(rng.uniform(-1, 1))
                a.I_priv = float(rng.choice([0.0, 1.0, 2.0]))
                a.mode = MODES[int(rng.integers(0, 4))]
                a.collected_r = float(rng.integers(0, 50))
                a.exploited_patch_id = int(rng.integers(-1, 3))
            a.soc_v_field = fields[i]
            rec["posx"][i, t], rec["posy"][i, t] = int(a.position[0]), int(a.position[1])
            rec["orientation"][i, t], rec["velocity"][i, t] = a.orientation, a.velocity
            rec["w"][i, t], rec["u"][i, t], rec["ipriv"][i, t] = a.w, a.u, a.I_priv
            rec["mode"][i, t] = MODES.index(a.mode)
            rec["collected"][i, t] = a.collected_r
            rec["patch_id"][i, t] = a.exploited_patch_id
            bits = np.packbits(fields[i].astype(np.uint8), bitorder="little")
            padded = np.zeros(words * 4, np.uint8)
            padded[: len(bits)] = bits
            soc[i, t] = padded.view("<u4")
        for k, r in enumerate(patches):
            if t == 0:
                r.position = np.array([float(rng.integers(30, 900)),
                                       float(rng.integers(30, 900))])
                r.resc_left = 100.0
            r.resc_left = float(r.resc_left - rng.choice([0.0, 0.5, 1.0]))
            r.unit_per_timestep = float(rng.uniform(0.1, 1.0))
            rec["res_posx"][k, t], rec["res_posy"][k, t] = int(r.position[0]), int(r.position[1])
            rec["res_left"][k, t], rec["res_quality"][k, t] = r.resc_left, r.unit_per_timestep
            rec["res_id"][k, t] = r.id
        ifdb.save_agent_data_RAM(agents, t + 1)
        ifdb.save_resource_data_RAM(patches, t + 1)
    agent_json = json.dumps(ifdb.agents_dict)
    store = {}
    sys.modules["zarr"] = _stub_zarr(store)
    ifdb.save_ifdb_as_csv(use_ram=True, as_zar=True, save_extracted_vfield=True)
    arrays = {name: {"shape": list(a.data.shape), "chunks": a.chunks, "dtype": a.data.dtype.str,
                     "data": a.data.tolist()} for name, a in store.items()}
    return {"rv": rv, "n": n, "n_patches": n_p, "steps": steps,
            "rec": {k: v.tolist() for k, v in rec.items()},
            "soc_bits": soc.astype(np.int64).tolist(),
            "radius": [float(r.radius) for r in patches],
            "agent_json": agent_json, "zarr": arrays}


def main(ref_root):
    import make_forage_golden
    make_forage_golden.install_foraging_shims(ref_root)
    from abm.monitoring import ifdb
    with tempfile.TemporaryDirectory() as tmp:   # the writer only creates this folder
        _cases(ifdb, tmp)


def _cases(ifdb, tmp):
    ifdb.importlib = types.SimpleNamespace(reload=lambda m: m)   # keep the settings below
    ifdb.ifdbp.TIMESTAMP_SAVE_DIR = tmp
    rng = np.random.default_rng(2027)
    rv = 70

    class Obj:
        pass

    out = {}
    # foraging agents and patches
    agents = [Obj() for _ in range(5)]
    for i, a in enumerate(agents):
        a.id = i
    patches = [Obj() for _ in range(2)]
    for k, r in enumerate(patches):
        r.id = k + 1
        r.radius = 30.0
    ifdb.ifdbp.envconf = {"VISUAL_FIELD_RESOLUTION": str(rv)}
    out["forage"] = _run(ifdb, agents, patches, 4, rv, rng, forage=True)
    # visual-flocking agents: the recorder's other fields keep Agent.__init__'s values
    agents = [Obj() for _ in range(6)]
    for i, a in enumerate(agents):
        a.id = i
        a.w, a.u, a.I_priv = 0, 0, 0
        a.mode, a.collected_r, a.exploited_patch_id = "explore", 0, -1
    out["vf"] = _run(ifdb, agents, [], 3, rv, rng, forage=False)
    with open(os.path.join(HERE, "recording_zarr.json"), "w") as f:
        json.dump(out, f)
    print("recording_zarr.json written to", HERE)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ABM_REFERENCE_ROOT")
    if not root:
        sys.exit(f"usage: python {os.path.basename(__file__)} REFERENCE_ROOT "
                 "(or set ABM_REFERENCE_ROOT): the root of the scioip34/ABM source tree")
    main(root)
