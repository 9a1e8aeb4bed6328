"""CPU-only checks of the C-ABI library: it loads, exports every entry point declared in
include/*.h, and its host-side logic (numpy-exact grids, defaults, argument validation) is
right.  No call here reaches a CUDA kernel."""
import ctypes
import math
import os
import re

import numpy as np
import pytest

from conftest import ROOT


@pytest.fixture(scope="module")
def lib():
    from abm_gb300 import _lib
    return _lib.load()


def declared_functions():
    names = set()
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(abm_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_exports_every_declared_symbol(lib):
    names = declared_functions()
    assert len(names) >= 10
    for name in names:
        assert hasattr(lib, name), name


def test_bindings_cover_header():
    from abm_gb300 import _lib
    bound = {s[0] for s in _lib.SIGNATURES}
    assert set(declared_functions()) <= bound


def test_abi_version(lib):
    assert lib.abm_vpf_abi_version() == 1


@pytest.mark.parametrize("rv", [8, 61, 122, 197, 333, 1200, 2666, 3600, 4999, 16384])
def test_phi_table_matches_numpy(lib, rv):
    ref = np.arange(-np.pi, np.pi, 2 * np.pi / rv)
    out = np.zeros(rv + 4)
    n = lib.abm_phi_table(rv, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), rv + 4)
    assert n == len(ref)
    assert np.array_equal(out[:n], ref)


def test_phi_mismatch_set_matches_numpy(lib):
    for rv in range(8, 5001):
        n = lib.abm_phi_table(rv, None, 0)
        assert n == len(np.arange(-np.pi, np.pi, 2 * np.pi / rv))


def test_words(lib):
    assert lib.abm_vpf_words(1200) == 38
    assert lib.abm_vpf_words(3600) == 113
    assert lib.abm_vpf_words(32) == 1
    assert lib.abm_vpf_words(0) < 0


def test_defaults_match_reference_vf_params(lib):
    from abm_gb300 import _lib
    p = _lib.AbmVfParams()
    assert lib.abm_vf_params_default(ctypes.byref(p)) == 0
    # vf_params.py:12-23 defaults; sims.py:60-61 geometry defaults
    assert (p.gam, p.v0, p.alp0, p.alp1, p.alp2) == (0.1, 1.0, 1.0, 0.09, 0.0)
    assert (p.bet0, p.bet1, p.bet2) == (1.0, 0.09, 0.0)
    assert (p.boundary, p.limit_movement, p.max_vel, p.max_th) == (0, 0, 3.0, 0.1)
    assert (p.width, p.height, p.window_pad, p.rv) == (600.0, 480.0, 30.0, 800)
    assert (p.fov0, p.fov1) == (-math.pi, math.pi)


def test_step_argument_validation(lib):
    """Invalid arguments are rejected before any CUDA call."""
    from abm_gb300 import _lib
    from abm_gb300.params import VFParams
    p = VFParams(rv=1).to_c()
    st = _lib.AbmSwarmState()
    r = lib.abm_vpf_flock_step(ctypes.byref(st), ctypes.byref(st), 10, ctypes.byref(p), None,
                               None, None, None, None)
    assert r == _lib.ABM_ERR_RV
    assert b"rv" in lib.abm_last_error_string()
    p = VFParams(rv=1200).to_c()
    r = lib.abm_vpf_flock_step(None, None, 10, ctypes.byref(p), None, None, None, None, None)
    assert r == _lib.ABM_ERR_INVALID_ARG
    r = lib.abm_vpf_flock_step(ctypes.byref(st), ctypes.byref(st), -1, ctypes.byref(p), None,
                               None, None, None, None)
    assert r == _lib.ABM_ERR_INVALID_ARG
    # n == 0 is a no-op
    assert lib.abm_vpf_flock_step(ctypes.byref(st), ctypes.byref(st), 0, ctypes.byref(p),
                                  None, None, None, None, None) == 0
    p.boundary = 7
    r = lib.abm_vpf_flock_step(ctypes.byref(st), ctypes.byref(st), 10, ctypes.byref(p), None,
                               None, None, None, None)
    assert r == _lib.ABM_ERR_INVALID_ARG
    p = VFParams(rv=1200, radius=0.0).to_c()
    r = lib.abm_vpf_flock_step(ctypes.byref(st), ctypes.byref(st), 10, ctypes.byref(p), None,
                               None, None, None, None)
    assert r == _lib.ABM_ERR_INVALID_ARG
    # aliasing in/out is refused
    buf = (ctypes.c_float * 4)()
    fp = ctypes.cast(buf, _lib.c_float_p)
    s = _lib.AbmSwarmState(fp, fp, fp, fp)
    p = VFParams(rv=1200).to_c()
    r = lib.abm_vpf_flock_step(ctypes.byref(s), ctypes.byref(s), 1, ctypes.byref(p), None,
                               None, None, None, None)
    assert r == _lib.ABM_ERR_INVALID_ARG


def test_record_argument_validation(lib):
    """The recorder and the recorded run reject invalid arguments before any CUDA call."""
    from abm_gb300 import _lib
    from abm_gb300.params import VFParams
    st = _lib.AbmSwarmState()
    step = (ctypes.c_int32 * 2)()
    sp = ctypes.cast(step, _lib.c_i32_p)
    rec = _lib.AbmVfRecording(4, sp, None, None, None, None, None)
    assert lib.abm_vpf_record(None, 1, None, 64, ctypes.byref(rec), None) == _lib.ABM_ERR_INVALID_ARG
    assert lib.abm_vpf_record(ctypes.byref(st), -1, None, 64, ctypes.byref(rec),
                              None) == _lib.ABM_ERR_INVALID_ARG
    # agents but no series
    assert lib.abm_vpf_record(ctypes.byref(st), 3, None, 64, ctypes.byref(rec),
                              None) == _lib.ABM_ERR_INVALID_ARG
    # a VPF series without the step's VPF, and a bad Rv for it
    buf = (ctypes.c_float * 4)()
    fp = ctypes.cast(buf, _lib.c_float_p)
    ibuf = (ctypes.c_int32 * 4)()
    ip = ctypes.cast(ibuf, _lib.c_i32_p)
    ubuf = (ctypes.c_uint32 * 4)()
    up = ctypes.cast(ubuf, _lib.c_u32_p)
    full = _lib.AbmSwarmState(fp, fp, fp, fp)
    rec = _lib.AbmVfRecording(4, sp, ip, ip, fp, fp, up)
    assert lib.abm_vpf_record(ctypes.byref(full), 1, None, 64, ctypes.byref(rec),
                              None) == _lib.ABM_ERR_INVALID_ARG
    assert lib.abm_vpf_record(ctypes.byref(full), 1, up, 0, ctypes.byref(rec),
                              None) == _lib.ABM_ERR_RV
    rec.step = None
    assert lib.abm_vpf_record(ctypes.byref(full), 1, up, 64, ctypes.byref(rec),
                              None) == _lib.ABM_ERR_INVALID_ARG
    p = VFParams(rv=64).to_c()
    assert lib.abm_vpf_flock_run_recorded(ctypes.byref(st), ctypes.byref(st), 1, ctypes.byref(p),
                                          None, 4, 2, None, None, None,
                                          None) == _lib.ABM_ERR_INVALID_ARG
    rec = _lib.AbmVfRecording(4, sp, ip, ip, fp, fp, up)
    assert lib.abm_vpf_flock_run_recorded(ctypes.byref(st), ctypes.byref(st), 1, ctypes.byref(p),
                                          None, 4, 2, None, ctypes.byref(rec), None,
                                          None) == _lib.ABM_ERR_INVALID_ARG


def test_step_config_validation(lib):
    assert lib.abm_vpf_set_step_config(3, 0) < 0
    assert lib.abm_vpf_set_step_config(0, 100) < 0
    w, t = ctypes.c_int32(), ctypes.c_int32()
    assert lib.abm_vpf_get_step_config(ctypes.byref(w), ctypes.byref(t)) == 0
    assert w.value in (1, 2, 4, 8, 16, 32) and t.value % 32 == 0


def test_params_from_env_gamma_quirk():
    from abm_gb300.params import VFParams
    env = {"VF_GAM": "0.5", "VF_ALP0": "2", "AGENT_FOV": "0.5",
           "VISUAL_FIELD_RESOLUTION": "1200", "BOUNDARY": "infinite"}
    p = VFParams.from_env(env)
    assert p.gam == 0.1          # vf_params.py:12 reads VF_GAMMA, the .env sets VF_GAM
    assert p.alp0 == 2.0 and p.boundary == "infinite"
    assert p.rv == 2400          # vf_sims.py:40-44 rescales Rv by 1/fov_ratio
    assert p.fov == (-0.5 * math.pi, 0.5 * math.pi)


def test_step_split_and_autotune_validation(lib):
    """Chunk counts other than 0 or a power of two up to 16 are refused; the autotuner
    rejects bad arguments before any CUDA call."""
    from abm_gb300 import _lib
    from abm_gb300.params import VFParams
    for bad in (-1, 3, 32):
        assert lib.abm_vpf_set_step_split(bad) == _lib.ABM_ERR_INVALID_ARG
    c = ctypes.c_int32()
    assert lib.abm_vpf_get_step_split(ctypes.byref(c)) == 0 and c.value in (0, 1, 2, 4, 8, 16)
    p = VFParams(rv=1200).to_c()
    st = _lib.AbmSwarmState()
    best = _lib.AbmStepConfig()
    seg = (ctypes.c_int32 * 2)()
    segp = ctypes.cast(seg, _lib.c_i32_p)
    calls = [  # (in, n, seg_begin, seg_end, params, reps, best)
        (None, 10, None, None, p, 3, best),
        (st, 0, None, None, p, 3, best),
        (st, 10, None, None, p, 0, best),
        (st, 10, segp, None, p, 3, best),
        (st, 10, None, None, p, 3, None),
    ]
    for s_in, n, sb, se, prm, reps, b in calls:
        r = lib.abm_vpf_autotune(ctypes.byref(s_in) if s_in is not None else None, n, sb, se,
                                 None, ctypes.byref(prm), None, reps,
                                 ctypes.byref(b) if b is not None else None, None, 0, None, None)
        assert r == _lib.ABM_ERR_INVALID_ARG
