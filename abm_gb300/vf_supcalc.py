"""Drop-in twins of the reference's visual-flocking math module.

Same names, signatures, argument meaning and return values as
``abm/projects/visual_flocking/vf_agent/vf_supcalc.py`` (scioip34/ABM 1.2.0):

* ``projection_field``                 vf_supcalc.py:20-138
* ``VSWRM_flocking_state_variables``   vf_supcalc.py:161-254

The arithmetic runs in the CUDA library (abm_vpf_project_rows / abm_vswrm_integrals); these
functions only marshal numpy arrays to the device and back.  For whole swarms use
``abm_gb300.swarm.VFSwarm``, which fuses both functions and the agent update into one launch.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib

_DEVICE = "cuda"


def _bits_from_field(V: np.ndarray) -> np.ndarray:
    """Binary field (raw pixel order) -> little-endian uint32 bitmask words."""
    b = np.packbits(np.asarray(V) > 0, bitorder="little")
    pad = (-len(b)) % 4
    if pad:
        b = np.concatenate([b, np.zeros(pad, np.uint8)])
    return b.view("<u4").astype(np.int32)


def projection_field(fov, v_field_resolution, position, radius, orientation,
                     object_positions, object_sizes=None, boundary_cond="walls",
                     arena_width=None, arena_height=None, vision_range=None, ag_id=0):
    """Visual projection field of one agent: (n objects, Rv) float64 of 0/1, flipped along
    the pixel axis exactly like the reference (vf_supcalc.py:134).  Objects at exactly the
    agent's position are skipped (:57-58).  Sizes are used as float32."""
    lib = _lib.load()
    rv = int(v_field_resolution)
    objs = np.asarray(object_positions, dtype=np.float64).reshape(-1, 2)
    n = objs.shape[0]
    if n == 0:
        return np.zeros((0, rv))
    dev = torch.device(_DEVICE)
    objs_d = torch.as_tensor(objs, device=dev).contiguous()
    sizes_d = None
    if object_sizes is not None:
        sizes_d = torch.as_tensor(np.asarray(object_sizes, np.float64), device=dev).contiguous()
    rows = torch.empty((n, rv), dtype=torch.float64, device=dev)
    fov_a = (ctypes.c_double * 2)(float(fov[0]), float(fov[1]))
    pos_a = (ctypes.c_double * 2)(float(position[0]), float(position[1]))
    stream = torch.cuda.current_stream(dev)
    status = lib.abm_vpf_project_rows(
        fov_a, rv, pos_a, float(radius), float(orientation), n, _lib.dptr(objs_d),
        _lib.dptr(sizes_d), 1 if boundary_cond == "infinite" else 0,
        float(arena_width or 0.0), float(arena_height or 0.0),
        -1.0 if vision_range is None else float(vision_range), _lib.dptr(rows), None,
        ctypes.c_void_p(stream.cuda_stream))
    _lib.check(status, "abm_vpf_project_rows")
    return rows.cpu().numpy()


def VSWRM_flocking_state_variables(vel_now, Phi, V_now, vf_params, t_now=None, V_prev=None,
                                   t_prev=None, verbose=False, ALP0=None, BET0=None, V0=None):
    """VSWRM increments (dvel, dpsi) of one agent from its binary VPF V_now (raw pixel order,
    paired with Phi); with verbose=True also (alpha_blob, alpha_edge, beta_blob, beta_edge).
    vf_params: any object with GAM, V0, ALP0, ALP1, ALP2, BET0, BET1, BET2."""
    out = vswrm_batch(np.asarray([vel_now], np.float64), Phi, np.asarray(V_now)[None, :],
                      vf_params, None if ALP0 is None else [ALP0],
                      None if BET0 is None else [BET0], None if V0 is None else [V0])[0]
    if not verbose:
        return float(out[0]), float(out[1])
    return tuple(float(v) for v in out)


def vswrm_batch(vel, Phi, V, vf_params, alp0=None, bet0=None, v0=None) -> np.ndarray:
    """Batched VSWRM_flocking_state_variables(verbose=True): (n, 6) float64."""
    lib = _lib.load()
    Phi = np.ascontiguousarray(Phi, dtype=np.float64)
    V = np.asarray(V)
    if V.ndim != 2 or V.shape[1] != Phi.shape[0]:
        # the reference's numpy broadcasting fails the same way (cos(Phi) * G_vel)
        raise ValueError(f"operands could not be broadcast together: Phi {Phi.shape}, "
                         f"V {V.shape}")
    n, rv = V.shape
    dev = torch.device(_DEVICE)
    bits = torch.as_tensor(np.stack([_bits_from_field(row) for row in V]), device=dev)
    vel_d = torch.as_tensor(np.asarray(vel, np.float32), device=dev).contiguous()
    ov = [None if a is None else torch.as_tensor(np.asarray(a, np.float32), device=dev)
          for a in (alp0, bet0, v0)]
    prm = (ctypes.c_double * 8)(*[float(getattr(vf_params, k)) for k in
                                  ("GAM", "V0", "ALP0", "ALP1", "ALP2", "BET0", "BET1",
                                   "BET2")])
    out = torch.empty((n, 6), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    status = lib.abm_vswrm_integrals(
        n, rv, _lib.u32ptr(bits), Phi.ctypes.data_as(_lib.c_double_p), _lib.fptr(vel_d), prm,
        *[_lib.fptr(t) for t in ov], _lib.dptr(out), ctypes.c_void_p(stream.cuda_stream))
    _lib.check(status, "abm_vswrm_integrals")
    return out.cpu().numpy()
