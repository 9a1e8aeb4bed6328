"""Recorded runs in the reference's on-disk layouts (host side of the device recorders).

The reference keeps every agent's per-step values in RAM (ifdb.save_agent_data_RAM /
save_resource_data_RAM, abm/monitoring/ifdb.py:55-96, :223-260) and writes them at the end of a
run with ifdb.save_ifdb_as_csv (ifdb.py:370-540): as agent_data.json / resource_data.json
(``as_zar=False``) or as zarr arrays ag_posx.zarr, ag_posy.zarr, ... of shape (agents, steps)
(``as_zar=True``, the setting of the shipped sweep experiments, ``USE_ZARR_FORMAT=1``), which
abm/loader/data_loader.py:83-93, :223-245 reads back.  The GPU recorders
(``abm_forage_record``, ``abm_vpf_record``) keep the same values as device series; this module
turns them into both layouts.

The zarr arrays are written in the zarr v2 storage format (a directory per array holding the
JSON metadata ``.zarray`` and one file per chunk named by its chunk indices joined with ".")
with uncompressed chunks (``"compressor": null``), which any zarr v2 reader accepts; the zarr
package itself is not needed.  The reference writes blosc-compressed chunks of the same arrays.
"""
from __future__ import annotations

import json
import os
import shutil

import numpy as np

# ifdb.mode_to_int (ifdb.py:197-206): the codes the recorders store
MODE_CODES = {"explore": 0, "exploit": 1, "relocate": 2, "collide": 3}


def _pad(number, n):
    """ifdb.pad_to_n_digits (ifdb.py:38-52)."""
    d = n - len(str(number))
    return d * "0" + str(number) if d > 0 else str(number)


def _fields(bits, rv, flip):
    """(steps, words) uint32 bitmasks -> (steps, rv) float64 0/1 fields."""
    by = np.ascontiguousarray(bits).astype("<u4").view(np.uint8).reshape(bits.shape[0], -1)
    f = np.unpackbits(by, axis=1, bitorder="little")[:, :rv].astype(np.float64)
    return f[:, ::-1] if flip else f


def agents_dict(rec: dict, rv: int, vpf_key: str = "soc_bits", flip: bool = False) -> dict:
    """The reference's agents_dict for a recording (ifdb.py:55-96): per agent id its name and
    per-step lists; the VPF stored as its rising and falling edge indices in numpy's printed
    form.  rec holds (n, steps) series posx, posy, orientation, velocity, w, u, ipriv, mode,
    collected, patch_id and, when present, rec[vpf_key] (n, steps, words) bitmasks (flip: the
    bitmask is in the reverse pixel order of the reference's field)."""
    n, steps = rec["posx"].shape
    bits = rec.get(vpf_key)
    words = bits.shape[2] if bits is not None and bits.ndim == 3 else 0
    out = {}
    for i in range(n):
        d = {"agent_name": f"agent-{_pad(i, 2)}",
             "posx": [int(v) for v in rec["posx"][i]], "posy": [int(v) for v in rec["posy"][i]],
             "orientation": [float(v) for v in rec["orientation"][i]],
             "velocity": [float(v) for v in rec["velocity"][i]],
             "w": [float(v) for v in rec["w"][i]], "u": [float(v) for v in rec["u"][i]],
             "Ipriv": [float(v) for v in rec["ipriv"][i]],
             "mode": [int(v) for v in rec["mode"][i]],
             "collectedr": [float(v) for v in rec["collected"][i]],
             "expl_patch_id": [int(v) for v in rec["patch_id"][i]],
             "vfield_up": [], "vfield_down": []}
        if words:
            for V in _fields(bits[i], rv, flip):
                d["vfield_up"].append(f"{np.where(np.roll(V, 1) < V)[0]}")
                d["vfield_down"].append(f"{np.where(np.roll(V, 1) > V)[0]}")
        out[i] = d
    return out


def resources_dict(rec: dict) -> dict:
    """The reference's resources_dict (ifdb.py:223-260): per patch id (in order of first
    appearance) its first step, name, per-step position / units left / quality and radius."""
    out = {}
    if "res_id" not in rec:
        return out
    steps = rec["res_id"].shape[1] if rec["res_id"].ndim == 2 else 0
    t0 = int(rec.get("t0", 0))
    for k in range(rec["res_id"].shape[0]):
        for t in range(steps):
            rid = int(rec["res_id"][k, t])
            if rid < 0:
                continue
            if rid not in out:
                out[rid] = {"start_time": t0 + t + 1, "end_time": None,
                            "res_name": f"res-{_pad(rid, 3)}", "pos_x": [], "pos_y": [],
                            "radius": int(rec["radius"][k]), "resc_left": [], "quality": []}
            r = out[rid]
            r["pos_x"].append(int(rec["res_posx"][k, t]))
            r["pos_y"].append(int(rec["res_posy"][k, t]))
            r["resc_left"].append(float(rec["res_left"][k, t]))
            r["quality"].append(float(rec["res_quality"][k, t]))
    return out


def reference_json(rec: dict, rv: int, vpf_key: str = "soc_bits", flip: bool = False):
    """(agent_data.json, resource_data.json) text exactly as json.dump writes the reference's
    dictionaries (ifdb.py:412-434)."""
    return (json.dumps(agents_dict(rec, rv, vpf_key, flip)), json.dumps(resources_dict(rec)))


def vf_series(rec: dict) -> dict:
    """A visual-flocking recording (posx, posy, orientation, velocity, optional vpf_bits) with
    the fields a VFAgent leaves at the values Agent.__init__ gives them (agent.py:68-126: w, u,
    I_priv 0, mode "explore", collected_r 0, exploited_patch_id -1), as the reference's recorder
    stores them for visual-flocking runs."""
    n, steps = rec["posx"].shape
    out = dict(rec)
    for k in ("w", "u", "ipriv", "collected"):
        out[k] = np.zeros((n, steps))
    out["mode"] = np.full((n, steps), MODE_CODES["explore"], np.int32)
    out["patch_id"] = np.full((n, steps), -1, np.int32)
    return out


# ---------------------------------------------------------------------------------- zarr v2
def write_zarr_array(path: str, data, chunks) -> None:
    """Write `data` as a zarr v2 array (float64 '<f8', C order, fill value 0.0) at the directory
    `path`, replacing what is there (zarr.open(path, mode='w', ...) then one assignment of the
    whole array); chunks are stored uncompressed, edge chunks padded to the full chunk shape."""
    data = np.ascontiguousarray(np.asarray(data, dtype="<f8"))
    chunks = tuple(int(c) for c in chunks)
    if len(chunks) != data.ndim or any(c < 1 for c in chunks):
        raise ValueError(f"chunks {chunks} do not fit an array of shape {data.shape}")
    if os.path.isdir(path):
        shutil.rmtree(path)
    os.makedirs(path)
    meta = {"chunks": list(chunks), "compressor": None, "dtype": "<f8", "fill_value": 0.0,
            "filters": None, "order": "C", "shape": list(data.shape), "zarr_format": 2}
    with open(os.path.join(path, ".zarray"), "w") as f:
        json.dump(meta, f, indent=4, sort_keys=True)
    grid = [-(-s // c) for s, c in zip(data.shape, chunks)]
    for idx in np.ndindex(*grid):
        sel = tuple(slice(i * c, min((i + 1) * c, s)) for i, c, s in zip(idx, chunks, data.shape))
        block = data[sel]
        if block.shape != chunks:
            full = np.zeros(chunks, "<f8")
            full[tuple(slice(0, b) for b in block.shape)] = block
            block = full
        with open(os.path.join(path, ".".join(str(i) for i in idx)), "wb") as f:
            f.write(np.ascontiguousarray(block).tobytes(order="C"))


def read_zarr_array(path: str) -> np.ndarray:
    """Read a zarr v2 array with uncompressed chunks (as write_zarr_array stores them); missing
    chunks read as the fill value."""
    with open(os.path.join(path, ".zarray")) as f:
        meta = json.load(f)
    if meta.get("zarr_format") != 2:
        raise ValueError(f"{path}: not a zarr v2 array")
    if meta.get("compressor") is not None or meta.get("filters"):
        raise ValueError(f"{path}: compressed or filtered chunks need the zarr package")
    dt = np.dtype(meta["dtype"])
    shape, chunks, order = tuple(meta["shape"]), tuple(meta["chunks"]), meta.get("order", "C")
    sep = meta.get("dimension_separator", ".")
    fill = meta.get("fill_value")
    out = np.full(shape, 0 if fill is None else fill, dt)
    grid = [-(-s // c) for s, c in zip(shape, chunks)]
    for idx in np.ndindex(*grid):
        fn = os.path.join(path, *([sep.join(str(i) for i in idx)] if sep == "." else
                                  [str(i) for i in idx]))
        if not os.path.exists(fn):
            continue
        with open(fn, "rb") as f:
            block = np.frombuffer(f.read(), dt).reshape(chunks, order=order)
        sel = tuple(slice(i * c, min((i + 1) * c, s)) for i, c, s in zip(idx, chunks, shape))
        out[sel] = block[tuple(slice(0, x.stop - x.start) for x in sel)]
    return out


def _edge_list(text: str):
    """The reference's parse of one stored edge string (ifdb.py:512-522): its spacing
    replacements, then json.loads and int(float(v)) of every element."""
    s = text.replace("   ", " ").replace("  ", " ").replace("[  ", "[").replace(
        "[ ", "[").replace(" ", ", ")
    return [int(float(v)) for v in json.loads(s)]


def reconstruct_vpf(rv: int, up, down) -> np.ndarray:
    """abm/loader/helper.py:39-52: ones on up[i]:down[i] for every i (Python slices, so a
    field whose run wraps around pixel 0 is not rebuilt as it was)."""
    if len(up) != len(down):
        raise Exception("Length of up and down edges differ during VPF reconstruction.")
    V = np.zeros(rv)
    for a, b in zip(up, down):
        V[a:b] = 1
    return V


def save_reference_zarr(folder: str, agents: dict, resources: dict, v_field_len=None,
                        save_extracted_vfield: bool = False) -> list:
    """Write the zarr arrays the reference's save_ifdb_as_csv(as_zar=True) writes for the
    "Base" project (ifdb.py:435-536) from its agents / resources dictionaries (agents_dict /
    resources_dict above): res_posx, res_posy, res_rad, res_left, res_qual (patches x steps)
    when there are patches; ag_posx, ag_posy, ag_ori, ag_vel, ag_mode, ag_w, ag_u, ag_ipriv,
    ag_collr, ag_explr (agents x steps); ag_vf (agents x steps x v_field_len, one chunk per step)
    when save_extracted_vfield.  Rows follow the reference's indexing: patch id p in row p - 1,
    agent id a in row a - 1, so agent 0 (ids start at 0) lands in the last row.  Returns the
    array names written."""
    os.makedirs(folder, exist_ok=True)
    written = []

    def put(name, arr, chunks):
        write_zarr_array(os.path.join(folder, name + ".zarr"), arr, chunks)
        written.append(name)

    num_res = len(resources)
    if num_res > 0:
        t_len = len(resources[next(iter(resources))]["pos_x"])
        cols = {"res_posx": "pos_x", "res_posy": "pos_y", "res_left": "resc_left",
                "res_qual": "quality"}
        arrs = {k: np.zeros((num_res, t_len)) for k in ("res_posx", "res_posy", "res_rad",
                                                        "res_left", "res_qual")}
        for rid, r in resources.items():
            for k, src in cols.items():
                arrs[k][rid - 1, :] = r[src]      # rows outside [-num_res, num_res) raise
            arrs["res_rad"][rid - 1, :] = [r["radius"] for _ in range(t_len)]
        for k in ("res_posx", "res_posy", "res_rad", "res_left", "res_qual"):
            put(k, arrs[k], (num_res, t_len))
    num_ag = len(agents)
    if num_ag == 0:
        raise ValueError("no agents recorded")
    t_len = len(agents[next(iter(agents))]["posx"])
    cols = {"ag_posx": "posx", "ag_posy": "posy", "ag_ori": "orientation", "ag_vel": "velocity",
            "ag_mode": "mode", "ag_w": "w", "ag_u": "u", "ag_ipriv": "Ipriv",
            "ag_collr": "collectedr", "ag_explr": "expl_patch_id"}
    arrs = {k: np.zeros((num_ag, t_len)) for k in cols}
    vf = None
    if v_field_len is not None and save_extracted_vfield:
        vf = np.zeros((num_ag, t_len, int(v_field_len)))
    for aid, d in agents.items():
        for k, src in cols.items():
            arrs[k][aid - 1, :] = d[src]
        if vf is not None:
            for t in range(t_len):
                up = _edge_list(d["vfield_up"][t])
                down = _edge_list(d["vfield_down"][t])
                vf[aid - 1, t, :] = (reconstruct_vpf(int(v_field_len), up, down) if up != []
                                     else np.zeros(int(v_field_len)))
    for k in cols:
        put(k, arrs[k], (num_ag, t_len))
    if vf is not None:
        put("ag_vf", vf, (num_ag, 1, int(v_field_len)))
    return written


def save_vf_run(folder: str, rec: dict, rv: int, as_zarr: bool = False, env=None,
                save_extracted_vfield: bool = False):
    """Save a visual-flocking recording (posx, posy, orientation, velocity and optionally
    vpf_bits in raw pixel order, (n, steps[, words])) like the end of VFSimulation.start
    (vf_sims.py:373-381): save_ifdb_as_csv as JSON or zarr, and env_params.json
    (env_saver.save_env_vars) when `env` is given."""
    if save_extracted_vfield and rec.get("vpf_bits") is None:
        raise ValueError("save_extracted_vfield needs the VPF in the recording "
                         "(record_steps(..., vpf=True))")
    os.makedirs(folder, exist_ok=True)
    series = vf_series(rec)
    if not as_zarr:
        agents, resources = reference_json(series, rv, "vpf_bits", flip=True)
        with open(os.path.join(folder, "agent_data.json"), "w") as f:
            f.write(agents)
        with open(os.path.join(folder, "resource_data.json"), "w") as f:
            f.write(resources)
    else:
        if not save_extracted_vfield:
            series = {k: v for k, v in series.items() if k != "vpf_bits"}
        save_reference_zarr(folder, agents_dict(series, rv, "vpf_bits", flip=True), {}, rv,
                            save_extracted_vfield)
    if env is not None:
        with open(os.path.join(folder, "env_params.json"), "w") as f:
            json.dump(dict(env), f, indent=4)
