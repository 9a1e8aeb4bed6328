"""Launch-configuration autotuner of the step (abm_vpf_autotune).

``tune(obj)`` times every candidate configuration of the step — the group form (4 focal
agents per warp) and the L1 form with 1, 2 or 4 warps per focal agent, each with 1-16
neighbour chunks, the tiled form with several agents-per-block
and tile lengths; for a batched sweep the L1 form with 1, 2 or 4 warps per agent — on the
object's own current state and stream, applies the fastest, and returns it with the whole
table.  All configurations give bit-identical results.  ``apply(config)`` re-applies a
configuration returned earlier (the library keeps one process-wide configuration).
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib

MAX_CANDIDATES = 64


def _target(obj):
    """(in-state struct, n, seg_begin, seg_end, order, params, overrides) of a VFSwarm or a
    BatchedSweep."""
    if hasattr(obj, "seg_begin"):   # BatchedSweep
        st = obj._state(obj._bufs[obj._cur])
        return st, obj.n, obj.seg_begin, obj.seg_end, obj.order, obj._cparams, obj._ov
    st = obj._state_struct(obj._cur)
    return st, obj.n, None, None, None, obj._cparams, obj._ov


def tune(obj, reps: int = 5, stream=None) -> dict:
    """Tune the step of `obj` (VFSwarm or BatchedSweep); returns {"best": {...},
    "tried": [{...}, ...]} with ms_per_step per configuration (-1: form refused)."""
    lib = _lib.load()
    st, n, sb, se, order, cparams, ov = _target(obj)
    s = stream if stream is not None else torch.cuda.current_stream(obj.device)
    best = _lib.AbmStepConfig()
    tried = (_lib.AbmStepConfig * MAX_CANDIDATES)()
    n_tried = ctypes.c_int32(0)
    status = lib.abm_vpf_autotune(ctypes.byref(st), int(n), _lib.i32ptr(sb), _lib.i32ptr(se),
                                  _lib.i32ptr(order), ctypes.byref(cparams), ctypes.byref(ov),
                                  int(reps), ctypes.byref(best), tried, MAX_CANDIDATES,
                                  ctypes.byref(n_tried), ctypes.c_void_p(s.cuda_stream))
    _lib.check(status, "abm_vpf_autotune")
    return {"best": best.as_dict(),
            "tried": [tried[k].as_dict() for k in range(min(n_tried.value, MAX_CANDIDATES))]}


def apply(config: dict) -> None:
    """Make `config` (a "best" entry of tune()) the library's step configuration."""
    lib = _lib.load()
    _lib.check(lib.abm_vpf_set_step_mode(int(config["mode"]), int(config["warps_per_agent"])))
    _lib.check(lib.abm_vpf_set_step_config(int(config["warps_per_block"]), int(config["tile"])))
    _lib.check(lib.abm_vpf_set_step_split(int(config["chunks"])))
