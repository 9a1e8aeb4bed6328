"""CPU check of the run recording's on-disk format: abm_gb300.foraging.reference_json writes
byte-for-byte the JSON the reference's own RAM recorder writes for the same states
(tests/golden/recording.json, make_recording_golden.py)."""
import json
import os

import numpy as np

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
