"""CPU parity oracle for the visual-flocking hot path (TEST INFRASTRUCTURE ONLY).

The oracle is an FP64 C restatement (``vpf_oracle.c``) of the reference functions

* ``vf_supcalc.projection_field``            abm/projects/visual_flocking/vf_agent/vf_supcalc.py:20-138
* ``vf_supcalc.calculate_closed_angle``      vf_supcalc.py:142-158
* ``vf_supcalc.VSWRM_flocking_state_variables`` / ``dPhi_V_of``  vf_supcalc.py:161-277
* ``VFAgent.calc_soc_v_proj`` / ``perform_action`` / ``update_agent_position``  vf_agent.py:216-327
* ``Agent.reflect_from_walls`` / ``prove_orientation``  abm/agent/agent.py:347-394, :605-610
* ``VFAgent.teleport_infinite_arena``       vf_agent.py:188-204
* ``Agent.calc_social_V_proj`` / ``projection_field`` / ``exlude_V_source_data``  agent.py:396-603
* ``supcalc.find_nearest`` / ``angle_between``  abm/agent/supcalc.py:8-34

wrapped here with ctypes.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline
leg of ``bench.py`` use it, always as the reference results or the timed CPU baseline; the library never
imports it.  It is pinned against fixtures produced by the reference itself
(``tests/golden/make_golden.py``) and the reference's own known-answer vectors.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "vpf_oracle.c")
_OUT_DIR = os.path.join(_HERE, "_build")
_LIB_PATH = os.path.join(_OUT_DIR, "liborc_vpf.so")
_lock = threading.Lock()
_lib = None

# Parameter slots of the oracle's double array (mirror abm_vf_params).
P_FIELDS = ["gam", "v0", "alp0", "alp1", "alp2", "bet0", "bet1", "bet2", "boundary",
            "limit_movement", "max_vel", "max_th", "width", "height", "window_pad", "fov0",
            "fov1", "rv", "radius", "dt"]


def build(force: bool = False) -> str:
    """Compile the oracle shared library (gcc, OpenMP when available)."""
    os.makedirs(_OUT_DIR, exist_ok=True)
    if (not force and os.path.exists(_LIB_PATH)
            and os.path.getmtime(_LIB_PATH) >= os.path.getmtime(_SRC)):
        return _LIB_PATH
    base = ["gcc", "-O3", "-fPIC", "-shared", "-ffp-contract=off", "-fno-fast-math"]
    tmp = _LIB_PATH + f".tmp{os.getpid()}"
    try:
        subprocess.run(base + ["-fopenmp", "-o", tmp, _SRC, "-lm"], check=True,
                       capture_output=True)
    except subprocess.CalledProcessError:
        subprocess.run(base + ["-o", tmp, _SRC, "-lm"], check=True, capture_output=True)
    os.replace(tmp, _LIB_PATH)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            path = build()
            L = ctypes.CDLL(path)
            dp = ctypes.POINTER(ctypes.c_double)
            ip = ctypes.POINTER(ctypes.c_int)
            u8p = ctypes.POINTER(ctypes.c_uint8)
            c_int, c_d = ctypes.c_int, ctypes.c_double
            L.orc_linspace.argtypes = [c_d, c_d, c_int, dp]
            L.orc_arange.argtypes = [c_d, c_d, c_d, dp, c_int]
            L.orc_arange.restype = c_int
            L.orc_find_nearest.argtypes = [dp, c_int, c_d]
            L.orc_find_nearest.restype = c_int
            L.orc_angle_between.argtypes = [c_d] * 4
            L.orc_angle_between.restype = c_d
            L.orc_closed_angle_vf.argtypes = [c_d] * 4
            L.orc_closed_angle_vf.restype = c_d
            L.orc_closed_angle_agent.argtypes = [c_d] * 4
            L.orc_closed_angle_agent.restype = c_d
            L.orc_projection_field.argtypes = [c_d, c_d, c_int, c_d, c_d, c_d, c_d, c_int, dp, dp,
                                               c_int, c_d, c_d, c_d, dp, dp]
            L.orc_projection_union.argtypes = [c_d, c_d, c_int, c_d, c_d, c_d, c_d, c_int, dp,
                                               dp, c_int, c_d, c_d, dp, dp]
            L.orc_projection_union_ex.argtypes = [c_d, c_d, c_int, c_d, c_d, c_d, c_d, c_int, dp,
                                                  dp, c_int, c_d, c_d, dp, dp, c_d, u8p, ip]
            L.orc_dphi_v.argtypes = [dp, c_int, dp]
            L.orc_vswrm.argtypes = [c_d, dp, dp, c_int, dp, c_d, c_d, c_d, dp]
            L.orc_vf_step.argtypes = [c_int, dp, dp, dp, dp, dp, dp, dp, dp, dp, c_int, dp, dp,
                                      dp, dp, u8p, dp, dp]
            L.orc_vf_step.restype = c_int
            L.orc_vf_step_range.argtypes = [c_int, c_int, c_int, dp, dp, dp, dp, dp, dp, dp, dp,
                                            dp, dp]
            L.orc_vf_step_range.restype = c_int
            L.orc_num_threads.restype = c_int
            L.orc_set_threads.argtypes = [c_int]
            L.orc_agent_projection_field.argtypes = [c_int, c_d, c_d, c_d, c_d, c_d, c_d, c_int,
                                                     c_int, dp, c_int, c_int, dp]
            L.orc_social_vpf.argtypes = [c_int, c_int, dp, dp, dp, dp, ip, ip, c_d, c_int, c_int,
                                         c_int, c_d, c_d, dp]
            L.orc_projection_excuse.argtypes = [c_d, c_d, c_int, c_d, c_d, c_d, c_d, c_int, dp,
                                                dp, c_int, c_d, c_d, c_d, c_d, c_int, u8p, ip]
            L.orc_vf_step_ex.argtypes = [c_int, dp, dp, dp, dp, dp, dp, dp, dp, dp, c_int, dp,
                                         dp, dp, dp, u8p, dp, dp, c_d, u8p, ip]
            L.orc_vf_step_ex.restype = c_int
            L.orc_np_mean.argtypes = [dp, ctypes.c_longlong, ctypes.c_longlong]
            L.orc_np_mean.restype = c_d
            _lib = L
    return _lib


def _dp(a):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def params_array(p) -> np.ndarray:
    """Pack a parameter mapping / object into the oracle's double array."""
    get = (lambda k: p[k]) if isinstance(p, dict) else (lambda k: getattr(p, k))
    return np.array([float(get(k)) for k in P_FIELDS], dtype=np.float64)


def linspace(rv: int) -> np.ndarray:
    out = np.empty(rv, np.float64)
    lib().orc_linspace(-np.pi, np.pi, rv, _dp(out))
    return out


def arange_phi(rv: int) -> np.ndarray:
    cap = rv + 8
    out = np.empty(cap, np.float64)
    n = lib().orc_arange(-np.pi, np.pi, (2 * np.pi) / rv, _dp(out), cap)
    return out[:n].copy()


def find_nearest(arr, value) -> int:
    a = _f64(arr)
    return int(lib().orc_find_nearest(_dp(a), len(a), float(value)))


def angle_between(v1, v2) -> float:
    return float(lib().orc_angle_between(float(v1[0]), float(v1[1]), float(v2[0]), float(v2[1])))


def calculate_closed_angle(v1, v2) -> float:
    return float(lib().orc_closed_angle_vf(float(v1[0]), float(v1[1]), float(v2[0]),
                                           float(v2[1])))


def projection_field(fov, v_field_resolution, position, radius, orientation, object_positions,
                     object_sizes=None, boundary_cond="walls", arena_width=None,
                     arena_height=None, vision_range=None, return_margins=False):
    """Oracle twin of vf_supcalc.projection_field (dense flipped rows)."""
    objs = _f64(np.asarray(object_positions, dtype=np.float64).reshape(-1, 2))
    n = objs.shape[0]
    sizes = None if object_sizes is None else _f64(np.asarray(object_sizes, np.float64))
    out = np.zeros((n, v_field_resolution), np.float64)
    marg = np.zeros(n, np.float64)
    lib().orc_projection_field(float(fov[0]), float(fov[1]), int(v_field_resolution),
                               float(position[0]), float(position[1]), float(radius),
                               float(orientation), n, _dp(objs), _dp(sizes),
                               1 if boundary_cond == "infinite" else 0,
                               float(arena_width or 0.0), float(arena_height or 0.0),
                               float("nan") if vision_range is None else float(vision_range),
                               _dp(out), _dp(marg))
    return (out, marg) if return_margins else out


def projection_union(fov, v_field_resolution, position, radius, orientation, object_positions,
                     object_sizes=None, infinite=False, arena_width=0.0, arena_height=0.0,
                     want_excuse=False, band=1e-9):
    """The OR of projection_field's rows in raw pixel order (calc_soc_v_proj's binarised sum,
    unflipped) without materialising the rows, and each object's decision margin; with
    want_excuse also the pixels (raw order) that objects within `band` rad of a pixel / width
    decision boundary can flip and the number of such objects."""
    objs = _f64(np.asarray(object_positions, dtype=np.float64).reshape(-1, 2))
    n = objs.shape[0]
    rv = int(v_field_resolution)
    sizes = None if object_sizes is None else _f64(np.asarray(object_sizes, np.float64))
    V = np.zeros(rv, np.float64)
    marg = np.zeros(n, np.float64)
    ex = np.zeros(rv, np.uint8) if want_excuse else None
    near = ctypes.c_int(0)
    lib().orc_projection_union_ex(
        float(fov[0]), float(fov[1]), rv, float(position[0]), float(position[1]),
        float(radius), float(orientation), n, _dp(objs), _dp(sizes), 1 if infinite else 0,
        float(arena_width), float(arena_height), _dp(V), _dp(marg), float(band),
        None if ex is None else ex.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
        ctypes.byref(near))
    if want_excuse:
        return V, marg, ex, int(near.value)
    return V, marg


def projection_excuse(fov, v_field_resolution, position, radius, orientation, object_positions,
                      object_sizes=None, boundary_cond="walls", arena_width=None,
                      arena_height=None, vision_range=None, band=1e-9):
    """Per object of projection_field: the pixels (flipped, like its rows) that the object's
    alternative pixel decisions would flip when its bearing or half angle lies within `band`
    rad of a decision boundary, and whether it does.  Returns (n x Rv uint8, n bool)."""
    objs = _f64(np.asarray(object_positions, dtype=np.float64).reshape(-1, 2))
    n = objs.shape[0]
    rv = int(v_field_resolution)
    sizes = None if object_sizes is None else _f64(np.asarray(object_sizes, np.float64))
    ex = np.zeros((n, rv), np.uint8)
    near = np.zeros(n, np.int32)
    lib().orc_projection_excuse(float(fov[0]), float(fov[1]), rv, float(position[0]),
                                float(position[1]), float(radius), float(orientation), n,
                                _dp(objs), _dp(sizes), 1 if boundary_cond == "infinite" else 0,
                                float(arena_width or 0.0), float(arena_height or 0.0),
                                float("nan") if vision_range is None else float(vision_range),
                                float(band), 1, ex.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)),
                                near.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return ex, near.astype(bool)


def dphi_v(V) -> np.ndarray:
    v = _f64(V)
    out = np.empty_like(v)
    lib().orc_dphi_v(_dp(v), len(v), _dp(out))
    return out


def vswrm(vel, Phi, V, params, alp0=None, bet0=None, v0=None) -> np.ndarray:
    """Oracle twin of VSWRM_flocking_state_variables(verbose=True): 6 values."""
    phi = _f64(Phi)
    v = _f64(V)
    P = params_array(params)
    out = np.empty(6, np.float64)
    nan = float("nan")
    lib().orc_vswrm(float(vel), _dp(phi), _dp(v), len(v), _dp(P),
                    nan if alp0 is None else float(alp0), nan if bet0 is None else float(bet0),
                    nan if v0 is None else float(v0), _dp(out))
    return out


def vf_step(state, params, radii=None, alp0=None, bet0=None, v0=None, sequential=False,
            want_vpf=True, want_terms=True, want_margins=False, want_excuse=False, band=1e-9):
    """One step of all agents; state = dict of float arrays x, y, theta, v.

    Returns dict with x, y, theta, v (new), vpf (n x Rv uint8 raw order), terms (n x 6),
    margins (n x n), phi_mismatch (bool); with want_excuse also excuse (n x Rv uint8 raw
    order: per agent the pixels its pairs within `band` rad of a pixel / width decision
    boundary can flip, the symmetric differences of their alternative decisions) and near
    (n: the number of such pairs per agent)."""
    x, y, th, v = (_f64(state[k]) for k in ("x", "y", "theta", "v"))
    n = len(x)
    P = params_array(params)
    rv = int(P[17])
    out = {k: np.empty(n, np.float64) for k in ("x", "y", "theta", "v")}
    vpf = np.zeros((n, rv), np.uint8) if want_vpf else None
    terms = np.zeros((n, 6), np.float64) if want_terms else None
    margins = np.full((n, n), np.inf) if want_margins else None
    excuse = np.zeros((n, rv), np.uint8) if want_excuse else None
    near = np.zeros(n, np.int32) if want_excuse else None
    r = _f64(radii)
    a0, b0, vv0 = _f64(alp0), _f64(bet0), _f64(v0)
    u8 = lambda a: None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    mism = lib().orc_vf_step_ex(
        n, _dp(x), _dp(y), _dp(th), _dp(v), _dp(r), _dp(P), _dp(a0), _dp(b0), _dp(vv0),
        1 if sequential else 0, _dp(out["x"]), _dp(out["y"]), _dp(out["theta"]),
        _dp(out["v"]), u8(vpf), _dp(terms), _dp(margins), float(band), u8(excuse),
        None if near is None else near.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    out.update(vpf=vpf, terms=terms, margins=margins, phi_mismatch=bool(mism))
    if want_excuse:
        out.update(excuse=excuse, near=near)
    return out


def vf_step_range(state, params, i0, i1, radii=None):
    """Snapshot step of focal agents [i0, i1) only (the bounded CPU-baseline sample)."""
    x, y, th, v = (_f64(state[k]) for k in ("x", "y", "theta", "v"))
    n = len(x)
    P = params_array(params)
    outs = [np.zeros(n, np.float64) for _ in range(4)]
    r = _f64(radii)
    lib().orc_vf_step_range(n, int(i0), int(i1), _dp(x), _dp(y), _dp(th), _dp(v), _dp(r),
                            _dp(P), *[_dp(o) for o in outs])
    return outs


def num_threads() -> int:
    return int(lib().orc_num_threads())


def set_threads(n: int) -> None:
    """Threads of the oracle's OpenMP loops from now on."""
    lib().orc_set_threads(int(n))


def agent_projection_field(rv, fov, position, radius, orientation, visual_exclusion,
                           social_xy, nonsocial_xy=None):
    """Oracle twin of Agent.projection_field(obstacles, non_expl_agents=...)."""
    soc = np.asarray(social_xy, np.float64).reshape(-1, 2)
    has_ns = nonsocial_xy is not None
    ns = np.asarray(nonsocial_xy if has_ns else np.zeros((0, 2)), np.float64).reshape(-1, 2)
    xy = _f64(np.concatenate([soc, ns], axis=0))
    out = np.zeros(rv, np.float64)
    lib().orc_agent_projection_field(int(rv), float(fov[0]), float(fov[1]), float(position[0]),
                                     float(position[1]), float(radius), float(orientation),
                                     1 if visual_exclusion else 0, xy.shape[0], _dp(xy),
                                     soc.shape[0], 1 if has_ns else 0, _dp(out))
    return out


def social_vpf(i, x, y, radii, theta, exploit, patch, vision_range, visual_exclusion,
               patchwise, rv, fov):
    """Oracle twin of Agent.calc_social_V_proj for focal agent i (flipped soc_v_field)."""
    n = len(x)
    xs, ys, rs, ts = (_f64(a) for a in (x, y, radii, theta))
    ex = np.ascontiguousarray(exploit, dtype=np.int32)
    pa = np.ascontiguousarray(patch, dtype=np.int32)
    out = np.zeros(rv, np.float64)
    ipt = ctypes.POINTER(ctypes.c_int)
    lib().orc_social_vpf(int(i), n, _dp(xs), _dp(ys), _dp(rs), _dp(ts),
                         ex.ctypes.data_as(ipt), pa.ctypes.data_as(ipt), float(vision_range),
                         1 if visual_exclusion else 0, 1 if patchwise else 0, int(rv),
                         float(fov[0]), float(fov[1]), _dp(out))
    return out


_FORAGER = (("x", np.float32), ("y", np.float32), ("theta", np.float32), ("v", np.float32),
            ("w", np.float64), ("u", np.float64), ("collected", np.float64),
            ("collected_before", np.float64), ("mode", np.int32), ("override_mode", np.int32),
            ("env_status", np.int32), ("env_status_before", np.int32),
            ("pool_success", np.int32), ("patch_id", np.int32), ("novelty", np.uint32),
            ("draws", np.uint64))
_PATCH = (("x", np.float64), ("y", np.float64), ("radius", np.float64), ("units", np.float64),
          ("left", np.float64), ("quality", np.float64), ("id", np.int32),
          ("draws", np.uint64))


def forage_step(agents, patches, fp, ip, seed, uniforms=None):
    """Oracle twin of abm_forage_step: returns (agents, patches, soc (n, rv) float64 stored
    order, failed regenerations); inputs are not modified.  fp, ip, seed: the arrays of
    ForageParams.oracle_arrays()."""
    a = {k: np.array(agents[k], dt, copy=True) for k, dt in _FORAGER}
    p = {k: np.array(patches[k], dt, copy=True) for k, dt in _PATCH}
    n, npch = len(a["x"]), len(p["x"])
    rv = int(ip[7])
    soc = np.zeros((n, rv), np.float64)
    fp = np.ascontiguousarray(fp, np.float64)
    # arrays without the collision switches (collide_agents, ghost_mode): collisions off
    ip = np.concatenate([np.asarray(ip, np.int32), np.array([0, 1], np.int32)[len(ip) - 10:]])
    ip = np.ascontiguousarray(ip, np.int32)
    uni = None if uniforms is None else np.ascontiguousarray(uniforms, np.float64)
    ptr = lambda arr: arr.ctypes.data_as(ctypes.c_void_p)
    failed = lib().orc_forage_step(
        n, *[ptr(a[k]) for k, _ in _FORAGER], npch, *[ptr(p[k]) for k, _ in _PATCH],
        ptr(fp), ptr(ip), ctypes.c_uint64(int(seed) & 0xFFFFFFFFFFFFFFFF),
        None if uni is None else ptr(uni), ptr(soc))
    return a, p, soc, int(failed)


def np_mean(a):
    """The oracle's restatement of np.mean over a float64 vector (pairwise summation)."""
    a = np.ascontiguousarray(a, np.float64)
    return float(lib().orc_np_mean(_dp(a), len(a), 1))


def philox4x32(ctr, key):
    """The oracle's Philox-4x32-10 block (four uint32 words)."""
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    out = (ctypes.c_uint32 * 4)()
    lib().orc_philox4x32(c, k, out)
    return [int(v) for v in out]
