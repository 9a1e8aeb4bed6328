"""ctypes bindings of ``libabm_vpf.so`` (declared in include/abm_vpf.h).

The library is the product: there is no CPU fallback.  Loading fails loudly when the
shared library is missing (build it with ``python -m abm_gb300._build``).
"""
from __future__ import annotations

import ctypes
import os
import threading

from . import _build

c_int32 = ctypes.c_int32
c_double = ctypes.c_double
c_void_p = ctypes.c_void_p
c_float_p = ctypes.POINTER(ctypes.c_float)
c_double_p = ctypes.POINTER(ctypes.c_double)
c_u32_p = ctypes.POINTER(ctypes.c_uint32)
c_u64_p = ctypes.POINTER(ctypes.c_ulonglong)
c_i32_p = ctypes.POINTER(ctypes.c_int32)

ABM_OK = 0
ABM_WARN_PHI_MISMATCH = 1
ABM_ERR_INVALID_ARG = -1
ABM_ERR_RV = -2
ABM_ERR_CUDA = -3
ABM_ERR_TIMEOUT = -4
ABM_ERR_NONFINITE = -5
ABM_ERR_UNSUPPORTED = -6
ABM_ERR_NO_DEVICE = -7
ABM_MAX_RV = 16384
ABM_NOALLOC_MAX_AGENTS = 65536
ABM_NOALLOC_MAX_RV = 8192
ABM_DIAG_COUNT = 8
DIAG_PAIRS_RESOLVED, DIAG_NEAR_BOUNDARY, DIAG_NONFINITE, DIAG_TIMEOUTS = 0, 1, 2, 3
DIAG_CAPACITY = 4


class AbmVfParams(ctypes.Structure):
    _fields_ = [("gam", c_double), ("v0", c_double), ("alp0", c_double), ("alp1", c_double),
                ("alp2", c_double), ("bet0", c_double), ("bet1", c_double), ("bet2", c_double),
                ("boundary", c_int32), ("limit_movement", c_int32), ("max_vel", c_double),
                ("max_th", c_double), ("width", c_double), ("height", c_double),
                ("window_pad", c_double), ("fov0", c_double), ("fov1", c_double),
                ("rv", c_int32), ("reserved0", c_int32), ("radius", c_double),
                ("dt", c_double)]


class AbmSwarmState(ctypes.Structure):
    _fields_ = [("x", c_float_p), ("y", c_float_p), ("theta", c_float_p), ("v", c_float_p)]


class AbmSwarmStateF64(ctypes.Structure):
    _fields_ = [("x", c_double_p), ("y", c_double_p), ("theta", c_double_p),
                ("v", c_double_p)]


class AbmAgentOverrides(ctypes.Structure):
    _fields_ = [("radius", c_float_p), ("alp0", c_float_p), ("bet0", c_float_p),
                ("v0", c_float_p)]


class AbmStepConfig(ctypes.Structure):
    _fields_ = [("mode", c_int32), ("warps_per_agent", c_int32), ("chunks", c_int32),
                ("warps_per_block", c_int32), ("tile", c_int32), ("ms_per_step", ctypes.c_float)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class AbmForageParams(ctypes.Structure):
    """abm_forage_params of include/abm_forage.h."""
    _fields_ = ([(k, ctypes.c_double) for k in ("T_w", "Eps_w", "g_w", "B_w", "w_max", "T_u",
                                                "Eps_u", "g_u", "B_u", "u_max", "S_wu",
                                                "S_uw", "F_N", "F_R")]
                + [("Tau", c_int32)]
                + [(k, ctypes.c_double) for k in ("exp_vel_max", "exp_theta_min",
                                                  "exp_theta_max", "reloc_theta_max",
                                                  "exp_stop_ratio", "width", "height",
                                                  "window_pad", "agent_radius", "consumption")]
                + [(k, c_int32) for k in ("pooling_time", "teleport_exploit",
                                          "regenerate_patches", "allow_border_patch_overlap",
                                          "min_resc_units", "max_resc_units")]
                + [(k, ctypes.c_double) for k in ("min_resc_quality", "max_resc_quality",
                                                  "patch_radius")]
                + [("rv", c_int32)]
                + [(k, ctypes.c_double) for k in ("fov0", "fov1", "vision_range")]
                + [(k, c_int32) for k in ("visual_exclusion", "patchwise_exclusion")]
                + [("seed", ctypes.c_uint64)]
                + [(k, c_int32) for k in ("collide_agents", "ghost_mode")])


# (field, pointer type) of abm_forager_state / abm_patch_state, in declaration order
FORAGER_FIELDS = (("x", c_float_p), ("y", c_float_p), ("theta", c_float_p), ("v", c_float_p),
                  ("w", c_double_p), ("u", c_double_p), ("collected", c_double_p),
                  ("collected_before", c_double_p), ("mode", c_i32_p),
                  ("override_mode", c_i32_p), ("env_status", c_i32_p),
                  ("env_status_before", c_i32_p), ("pool_success", c_i32_p),
                  ("patch_id", c_i32_p), ("novelty", c_u32_p), ("draws", c_u64_p),
                  ("ipriv", c_double_p))
PATCH_FIELDS = (("x", c_double_p), ("y", c_double_p), ("radius", c_double_p),
                ("units", c_double_p), ("left", c_double_p), ("quality", c_double_p),
                ("id", c_i32_p), ("draws", c_u64_p))


# (field, pointer type) of abm_forage_recording after its capacity and step counter
RECORDING_FIELDS = (("posx", c_i32_p), ("posy", c_i32_p), ("orientation", c_float_p),
                    ("velocity", c_float_p), ("w", c_double_p), ("u", c_double_p),
                    ("ipriv", c_double_p), ("collected", c_double_p), ("mode", c_i32_p),
                    ("patch_id", c_i32_p), ("soc_bits", c_u32_p), ("res_posx", c_i32_p),
                    ("res_posy", c_i32_p), ("res_left", c_double_p),
                    ("res_quality", c_double_p), ("res_id", c_i32_p))


class AbmForageRecording(ctypes.Structure):
    _fields_ = [("capacity", c_int32), ("step", c_i32_p)] + list(RECORDING_FIELDS)


class AbmVfRecording(ctypes.Structure):
    _fields_ = [("capacity", c_int32), ("step", c_i32_p), ("posx", c_i32_p), ("posy", c_i32_p),
                ("orientation", c_float_p), ("velocity", c_float_p), ("vpf_bits", c_u32_p)]


class AbmForagerState(ctypes.Structure):
    _fields_ = list(FORAGER_FIELDS)


class AbmPatchState(ctypes.Structure):
    _fields_ = list(PATCH_FIELDS)


# (name, restype, argtypes) of every exported entry point of include/abm_vpf.h and
# include/abm_forage.h
SIGNATURES = [
    ("abm_vpf_abi_version", c_int32, []),
    ("abm_last_error_string", ctypes.c_char_p, []),
    ("abm_vf_params_default", c_int32, [ctypes.POINTER(AbmVfParams)]),
    ("abm_phi_table", c_int32, [c_int32, c_double_p, c_int32]),
    ("abm_vpf_words", c_int32, [c_int32]),
    ("abm_vpf_flock_step", c_int32,
     [ctypes.POINTER(AbmSwarmState), ctypes.POINTER(AbmSwarmState), c_int32,
      ctypes.POINTER(AbmVfParams), ctypes.POINTER(AbmAgentOverrides), c_u32_p, c_double_p,
      c_u64_p, c_void_p]),
    ("abm_vpf_flock_batched", c_int32,
     [ctypes.POINTER(AbmSwarmState), ctypes.POINTER(AbmSwarmState), c_int32, c_i32_p, c_i32_p,
      c_i32_p, ctypes.POINTER(AbmVfParams), ctypes.POINTER(AbmAgentOverrides), c_u32_p,
      c_double_p, c_u64_p, c_void_p]),
    ("abm_vpf_flock_run", c_int32,
     [ctypes.POINTER(AbmSwarmState), ctypes.POINTER(AbmSwarmState), c_int32,
      ctypes.POINTER(AbmVfParams), ctypes.POINTER(AbmAgentOverrides), c_int32, c_int32, c_u64_p,
      c_void_p]),
    ("abm_vpf_flock_batched_run", c_int32,
     [ctypes.POINTER(AbmSwarmState), ctypes.POINTER(AbmSwarmState), c_int32, c_i32_p, c_i32_p,
      c_i32_p, ctypes.POINTER(AbmVfParams), ctypes.POINTER(AbmAgentOverrides), c_int32, c_int32,
      c_u64_p, c_void_p]),
    ("abm_vpf_flock_step_noalloc", c_int32,
     [ctypes.POINTER(AbmSwarmState), ctypes.POINTER(AbmSwarmState), c_int32,
      ctypes.POINTER(AbmVfParams), ctypes.POINTER(AbmAgentOverrides), c_u32_p, c_double_p,
      c_u64_p, c_void_p]),
    ("abm_vpf_project_rows", c_int32,
     [c_double_p, c_int32, c_double_p, c_double, c_double, c_int32, c_double_p, c_double_p,
      c_int32, c_double, c_double, c_double, c_double_p, c_u64_p, c_void_p]),
    ("abm_vswrm_integrals", c_int32,
     [c_int32, c_int32, c_u32_p, c_double_p, c_float_p, c_double_p, c_float_p, c_float_p,
      c_float_p, c_double_p, c_void_p]),
    ("abm_vpf_social_fields", c_int32,
     [c_float_p, c_float_p, c_float_p, c_float_p, c_double, c_i32_p, c_i32_p, c_int32, c_double,
      c_int32, c_int32, c_int32, c_double, c_double, c_u32_p, c_u64_p, c_void_p]),
    ("abm_vpf_edge_fwd", c_int32,
     [ctypes.POINTER(AbmSwarmState), ctypes.POINTER(AbmSwarmState), c_int32,
      ctypes.POINTER(AbmVfParams), c_int32, c_float_p, c_void_p]),
    ("abm_vpf_edge_bwd", c_int32,
     [ctypes.POINTER(AbmSwarmState), ctypes.POINTER(AbmSwarmState),
      ctypes.POINTER(AbmSwarmState), c_double_p, c_int32, ctypes.POINTER(AbmVfParams), c_int32,
      c_void_p]),
    ("abm_vpf_edge_fwd_f64", c_int32,
     [ctypes.POINTER(AbmSwarmStateF64), ctypes.POINTER(AbmSwarmStateF64), c_int32,
      ctypes.POINTER(AbmVfParams), c_int32, c_double_p, c_void_p]),
    ("abm_vpf_edge_bwd_f64", c_int32,
     [ctypes.POINTER(AbmSwarmStateF64), ctypes.POINTER(AbmSwarmStateF64),
      ctypes.POINTER(AbmSwarmStateF64), c_double_p, c_int32, ctypes.POINTER(AbmVfParams),
      c_int32, c_void_p]),
    ("abm_vpf_set_step_config", c_int32, [c_int32, c_int32]),
    ("abm_vpf_get_step_config", c_int32, [c_i32_p, c_i32_p]),
    ("abm_vpf_set_step_mode", c_int32, [c_int32, c_int32]),
    ("abm_vpf_get_step_mode", c_int32, [c_i32_p, c_i32_p]),
    ("abm_vpf_set_step_split", c_int32, [c_int32]),
    ("abm_vpf_get_step_split", c_int32, [c_i32_p]),
    ("abm_vpf_polarisation", c_int32,
     [c_float_p, c_int32, c_i32_p, c_int32, c_double_p, c_int32, c_i32_p, ctypes.c_void_p]),
    ("abm_vpf_flock_run_recorded", c_int32,
     [ctypes.POINTER(AbmSwarmState), ctypes.POINTER(AbmSwarmState), c_int32,
      ctypes.POINTER(AbmVfParams), ctypes.POINTER(AbmAgentOverrides), c_int32, c_int32, c_u32_p,
      ctypes.POINTER(AbmVfRecording), c_u64_p, ctypes.c_void_p]),
    ("abm_vpf_record", c_int32,
     [ctypes.POINTER(AbmSwarmState), c_int32, c_u32_p, c_int32, ctypes.POINTER(AbmVfRecording),
      ctypes.c_void_p]),
    ("abm_vpf_flock_step_host", c_int32,
     [ctypes.POINTER(AbmSwarmState), ctypes.POINTER(AbmSwarmState), c_int32,
      ctypes.POINTER(AbmVfParams), ctypes.POINTER(AbmAgentOverrides), ctypes.c_void_p]),
    ("abm_forage_params_default", c_int32, [ctypes.POINTER(AbmForageParams)]),
    ("abm_forage_run", c_int32,
     [ctypes.POINTER(AbmForagerState), c_int32, ctypes.POINTER(AbmPatchState), c_int32,
      ctypes.POINTER(AbmForageParams), c_u32_p, c_i32_p, c_int32, c_int32,
      ctypes.POINTER(AbmForageRecording), c_u64_p, ctypes.c_void_p]),
    ("abm_forage_step", c_int32,
     [ctypes.POINTER(AbmForagerState), c_int32, ctypes.POINTER(AbmPatchState), c_int32,
      ctypes.POINTER(AbmForageParams), c_u32_p, c_i32_p, c_double_p, c_u64_p, ctypes.c_void_p]),
    ("abm_forage_record", c_int32,
     [ctypes.POINTER(AbmForagerState), c_int32, ctypes.POINTER(AbmPatchState), c_int32, c_u32_p,
      c_int32, ctypes.POINTER(AbmForageRecording), ctypes.c_void_p]),
    ("abm_philox4x32", None, [ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_uint32),
                              ctypes.POINTER(ctypes.c_uint32)]),
    ("abm_vpf_autotune", c_int32,
     [ctypes.POINTER(AbmSwarmState), c_int32, c_i32_p, c_i32_p, c_i32_p,
      ctypes.POINTER(AbmVfParams), ctypes.POINTER(AbmAgentOverrides), c_int32,
      ctypes.POINTER(AbmStepConfig), ctypes.POINTER(AbmStepConfig), c_int32, c_i32_p,
      ctypes.c_void_p]),
    ("abm_vpf_check_sincos", c_int32, [c_float_p, c_int32, c_double_p, c_void_p]),
    ("abm_vpf_status", c_int32, [c_int32, c_void_p]),
    ("abm_vpf_debug_wait_timeout", c_int32, [c_int32, c_u64_p, c_i32_p, c_void_p]),
    ("abm_probe_pipe_peak", c_int32,
     [c_int32, c_int32, c_int32, c_int32, c_float_p, c_double_p, c_void_p]),
]

_lock = threading.Lock()
_lib = None


class AbmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"abm_vpf error {code}: {msg}")
        self.code = code


def lib_path() -> str:
    return _build.LIB_PATH


def load(build_if_missing: bool = True):
    """Load (building first if needed and allowed) the CUDA library."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIB_PATH
        if build_if_missing:
            path = _build.build()
        if not os.path.exists(path):
            raise RuntimeError(f"abm_gb300 CUDA library not found at {path}; "
                               "run `python -m abm_gb300._build`")
        L = ctypes.CDLL(path)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


def check(status: int, what: str = "") -> int:
    """Raise AbmError on a negative status; return warnings (positive) unchanged."""
    if status < 0:
        msg = load().abm_last_error_string().decode(errors="replace")
        raise AbmError(status, f"{what}: {msg}" if what else msg)
    return status


def fptr(t):
    """float* of a contiguous float32 torch tensor (or None)."""
    if t is None:
        return None
    return ctypes.cast(t.data_ptr(), c_float_p)


def dptr(t):
    if t is None:
        return None
    return ctypes.cast(t.data_ptr(), c_double_p)


def u32ptr(t):
    if t is None:
        return None
    return ctypes.cast(t.data_ptr(), c_u32_p)


def i32ptr(t):
    if t is None:
        return None
    return ctypes.cast(t.data_ptr(), c_i32_p)


def u64ptr(t):
    if t is None:
        return None
    return ctypes.cast(t.data_ptr(), c_u64_p)
