"""Generate tests/golden/metarunner.json with the REFERENCE's MetaProtocol.

    PYTHONDONTWRITEBYTECODE=1 python tests/golden/make_metarunner_golden.py /path/to/reference

For several sweep definitions (linspace ranges, explicit values, booleans, product and
quadratic restraints) the reference's own Tunable / Constant / TunedPairRestrain objects are
added to a MetaProtocol, and the combinations are computed the way generate_temp_env_files
does (itertools.product over the criteria, then MetaProtocol.consider_tuned_pairs,
abm/metarunner/metarunner.py:136-189); nothing is written to disk by the reference (its own
env-file writer is not called).
"""
import contextlib
import io
import itertools
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

CASES = [
    {"criteria": [["Tunable", "VF_ALP0", 0.1, 3.0, 5], ["Tunable", "VF_BET0", [0.5, 1, 2]],
                  ["Constant", "N", 20]], "pairs": [], "qpairs": []},
    {"criteria": [["Tunable", "VF_ALP0", [0.5, 1, 2]], ["Tunable", "VF_BET0", [0.5, 1, 2]]],
     "pairs": [["VF_ALP0", "VF_BET0", 1.0]], "qpairs": []},
    {"criteria": [["Tunable", "VF_ALP1", [0.5, 2.0, 0.125]], ["Tunable", "VF_BET1", [1.0, 0.5, 2.0]],
                  ["Constant", "VF_ALP0", 1.0]], "pairs": [], "qpairs": [["VF_ALP1", "VF_BET1", 0.5]]},
    {"criteria": [["Tunable", "AGENT_AGENT_COLLISION", [True, False]],
                  ["Tunable", "N", 5, 25, 3]], "pairs": [], "qpairs": []},
    {"criteria": [["Tunable", "VF_ALP0", 0.0, 1.0, 4], ["Tunable", "VF_BET0", 0.0, 2.0, 3],
                  ["Tunable", "VF_V0", [1, 2]]],
     "pairs": [["VF_ALP0", "VF_BET0", 0.0]], "qpairs": [["VF_V0", "VF_ALP0", 0.0]]},
]


def build(mr, case):
    mp = object.__new__(mr.MetaProtocol)
    mp.tunables, mp.tuned_pairs, mp.q_tuned_pairs = [], [], []
    for c in case["criteria"]:
        if c[0] == "Constant":
            mp.tunables.append(mr.Constant(c[1], c[2]))
        elif isinstance(c[2], list):
            mp.tunables.append(mr.Tunable(c[1], values_override=c[2]))
        else:
            mp.tunables.append(mr.Tunable(c[1], min_v=c[2], max_v=c[3], num_data_points=c[4]))
    for a, b, v in case["pairs"]:
        mp.tuned_pairs.append(mr.TunedPairRestrain(a, b, v))
    for a, b, v in case["qpairs"]:
        mp.q_tuned_pairs.append(mr.TunedPairRestrain(a, b, v))
    return mp


def main(ref_root):
    import types
    import make_forage_golden
    make_forage_golden.install_foraging_shims(ref_root)

    class _Mod(types.ModuleType):
        def __getattr__(self, k):
            return type(k, (), {"__init__": lambda s, *a, **kw: None})

    # metarunner imports abm.app only to start simulations (run_protocol), not used here
    import abm
    sys.modules["abm.app"] = _Mod("abm.app")
    abm.app = sys.modules["abm.app"]
    from abm.metarunner import metarunner as mr
    out = []
    for case in CASES:
        mp = build(mr, case)
        combos = list(itertools.product(*[t.get_values() for t in mp.tunables]))
        with contextlib.redirect_stdout(io.StringIO()):
            kept = mp.consider_tuned_pairs(combos)
        out.append(dict(case, combos=[[float(v) if not isinstance(v, bool) else bool(v)
                                       for v in c] for c in kept]))
    with open(os.path.join(HERE, "metarunner.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("metarunner.json written to", HERE)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ABM_REFERENCE_ROOT")
    if not root:
        sys.exit(f"usage: python {os.path.basename(__file__)} REFERENCE_ROOT "
                 "(or set ABM_REFERENCE_ROOT): the root of the scioip34/ABM source tree")
    main(root)
