"""CPU check of the run recording's on-disk format: abm_gb300.foraging.reference_json writes
byte-for-byte the JSON the reference's own RAM recorder writes for the same states
(tests/golden/recording.json, make_recording_golden.py)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN


def test_reference_json_matches_reference_recorder():
    from abm_gb300.foraging import reference_json
    d = json.load(open(os.path.join(GOLDEN, "recording.json")))
    r = d["rec"]
    rec = {"posx": np.array(r["posx"], np.int32), "posy": np.array(r["posy"], np.int32),
           "orientation": np.array(r["orientation"], np.float32),
           "velocity": np.array(r["velocity"], np.float32),
           "w": np.array(r["w"]), "u": np.array(r["u"]), "ipriv": np.array(r["ipriv"]),
           "collected": np.array(r["collected"]), "mode": np.array(r["mode"], np.int32),
           "patch_id": np.array(r["patch_id"], np.int32),
           "res_posx": np.array(r["res_posx"], np.int32),
           "res_posy": np.array(r["res_posy"], np.int32),
           "res_left": np.array(r["res_left"]), "res_quality": np.array(r["res_quality"]),
           "res_id": np.array(r["res_id"], np.int32),
           "soc_bits": np.array(d["soc_bits"], np.int64).astype(np.uint32),
           "radius": np.array(d["radius"]), "t0": 0}
    agents, resources = reference_json(rec, d["rv"])
    assert agents == d["agent_json"]
    assert resources == d["resource_json"]


def _zarr_case(name):
    d = json.load(open(os.path.join(GOLDEN, "recording_zarr.json")))[name]
    r = d["rec"]
    rec = {k: np.array(v) for k, v in r.items()}
    for k in ("posx", "posy", "mode", "patch_id", "res_posx", "res_posy", "res_id"):
        rec[k] = rec[k].astype(np.int32)
    for k in ("orientation", "velocity"):
        rec[k] = rec[k].astype(np.float32)
    rec["soc_bits"] = np.array(d["soc_bits"], np.int64).astype(np.uint32)
    rec["radius"] = np.array(d["radius"])
    rec["t0"] = 0
    return d, rec


def _check_zarr_folder(folder, expected):
    from abm_gb300.recording import read_zarr_array
    names = sorted(n for n in os.listdir(folder) if n.endswith(".zarr"))
    assert names == sorted(expected)
    for name, exp in expected.items():
        meta = json.load(open(os.path.join(folder, name, ".zarray")))
        assert meta["shape"] == exp["shape"] and meta["chunks"] == exp["chunks"]
        assert meta["dtype"] == exp["dtype"] == "<f8"
        got = read_zarr_array(os.path.join(folder, name))
        np.testing.assert_array_equal(got, np.array(exp["data"]), err_msg=name)


def test_zarr_arrays_match_reference_writer(tmp_path):
    """Foraging run: the arrays of save_ifdb_as_csv(as_zar=True, save_extracted_vfield=True)
    as the reference's own writer fills them (row id - 1, agent 0 in the last row, ag_vf
    rebuilt by reconstruct_VPF from the stored edge strings)."""
    from abm_gb300.recording import agents_dict, resources_dict, save_reference_zarr
    d, rec = _zarr_case("forage")
    save_reference_zarr(str(tmp_path), agents_dict(rec, d["rv"]), resources_dict(rec), d["rv"],
                        save_extracted_vfield=True)
    _check_zarr_folder(str(tmp_path), d["zarr"])
    assert json.dumps(agents_dict(rec, d["rv"])) == d["agent_json"]


def _raw_vpf_bits(soc_bits, rv):
    """The reference's soc_v_field bitmasks -> the raw pixel order the flocking step writes."""
    n, steps, words = soc_bits.shape
    by = soc_bits.astype("<u4").view(np.uint8).reshape(n, steps, -1)
    f = np.unpackbits(by, axis=2, bitorder="little")[:, :, :rv][:, :, ::-1]
    packed = np.packbits(np.ascontiguousarray(f), axis=2, bitorder="little")
    out = np.zeros((n, steps, words * 4), np.uint8)
    out[:, :, : packed.shape[2]] = packed
    return out.view("<u4").astype(np.uint32)


def test_vf_run_json_and_zarr_match_reference_writer(tmp_path):
    """Visual-flocking run: the recorder's other fields at Agent.__init__'s values, the VPF
    given in the step's raw pixel order (the reference's field is its flip)."""
    from abm_gb300.recording import save_vf_run
    d, rec = _zarr_case("vf")
    vf = {k: rec[k] for k in ("posx", "posy", "orientation", "velocity")}
    vf["vpf_bits"] = _raw_vpf_bits(rec["soc_bits"], d["rv"])
    save_vf_run(str(tmp_path / "json"), vf, d["rv"], as_zarr=False, env={"N": "6"})
    assert open(tmp_path / "json" / "agent_data.json").read() == d["agent_json"]
    assert open(tmp_path / "json" / "resource_data.json").read() == "{}"
    assert json.load(open(tmp_path / "json" / "env_params.json")) == {"N": "6"}
    save_vf_run(str(tmp_path / "zarr"), vf, d["rv"], as_zarr=True, save_extracted_vfield=True)
    _check_zarr_folder(str(tmp_path / "zarr"), d["zarr"])
    save_vf_run(str(tmp_path / "plain"), vf, d["rv"], as_zarr=True)
    _check_zarr_folder(str(tmp_path / "plain"),
                       {k: v for k, v in d["zarr"].items() if k != "ag_vf.zarr"})
    no_vpf = {k: v for k, v in vf.items() if k != "vpf_bits"}
    with pytest.raises(ValueError):
        save_vf_run(str(tmp_path / "bad"), no_vpf, d["rv"], as_zarr=True,
                    save_extracted_vfield=True)


def test_zarr_v2_store_layout(tmp_path):
    """The zarr v2 directory layout: .zarray metadata, one uncompressed C-order chunk file per
    chunk named by its indices, edge chunks padded to the full chunk shape."""
    from abm_gb300.recording import read_zarr_array, write_zarr_array
    rng = np.random.default_rng(5)
    a = rng.standard_normal((5, 7, 3))
    p = str(tmp_path / "a.zarr")
    write_zarr_array(p, a, (2, 1, 3))
    meta = json.load(open(os.path.join(p, ".zarray")))
    assert meta == {"chunks": [2, 1, 3], "compressor": None, "dtype": "<f8", "fill_value": 0.0,
                    "filters": None, "order": "C", "shape": [5, 7, 3], "zarr_format": 2}
    files = sorted(f for f in os.listdir(p) if f != ".zarray")
    assert files == sorted(f"{i}.{j}.0" for i in range(3) for j in range(7))
    edge = np.frombuffer(open(os.path.join(p, "2.4.0"), "rb").read(), "<f8").reshape(2, 1, 3)
    np.testing.assert_array_equal(edge[0], a[4:5, 4])
    np.testing.assert_array_equal(edge[1], 0.0)
    np.testing.assert_array_equal(read_zarr_array(p), a)
    write_zarr_array(p, a[:2, :2, :1], (2, 2, 1))       # mode 'w' replaces the array
    assert sorted(f for f in os.listdir(p) if f != ".zarray") == ["0.0.0"]


def test_edge_string_parse_round_trip():
    """The reference's parse of the stored edge strings (replacements + json.loads) recovers
    the edge indices, also when numpy wraps the printed array over several lines."""
    from abm_gb300.recording import _edge_list, reconstruct_vpf
    rng = np.random.default_rng(9)
    for rv in (40, 1200, 3600):
        V = (rng.random(rv) < 0.4).astype(np.float64)
        V[0] = V[-1] = 0.0     # no run touches the ends (those pair their edges wrongly)
        up = np.where(np.roll(V, 1) < V)[0]
        down = np.where(np.roll(V, 1) > V)[0]
        assert len(up) < 1000
        assert _edge_list(f"{up}") == up.tolist()
        assert _edge_list(f"{down}") == down.tolist()
        np.testing.assert_array_equal(reconstruct_vpf(rv, up, down), V)
