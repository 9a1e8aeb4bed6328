"""Foraging social VPF channel (the reference's Agent.calc_social_V_proj, abm/agent/agent.py:396-419).

``social_fields`` computes, for every agent, the projection field of the exploiting agents in
vision range with the reference's distance-ordered visual exclusion, in the stored order of
the reference's ``soc_v_field`` (flipped and FOV-masked), through abm_vpf_social_fields.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from . import _lib


def social_fields(x, y, theta, exploit, patch, vision_range, visual_exclusion=True,
                  patchwise=True, rv=1200, fov=(-math.pi, math.pi), radius=10.0, radii=None,
                  device="cuda", diag=None, as_bits=False):
    """x, y: top-left positions; exploit: nonzero where the agent's mode is "exploit";
    patch: exploited patch id (-1 for none).  Returns (n, rv) uint8 (or the raw bitmask words
    when as_bits=True, as an int32 device tensor)."""
    lib = _lib.load()
    dev = torch.device(device)
    f = lambda a: torch.as_tensor(np.asarray(a, np.float32) if not torch.is_tensor(a) else a,
                                  dtype=torch.float32, device=dev).contiguous()
    i32 = lambda a: torch.as_tensor(np.asarray(a, np.int32) if not torch.is_tensor(a) else a,
                                    dtype=torch.int32, device=dev).contiguous()
    xs, ys, ts = f(x), f(y), f(theta)
    ex, pa = i32(exploit), i32(patch)
    rs = None if radii is None else f(radii)
    n = xs.numel()
    words = (int(rv) + 31) // 32
    out = torch.zeros((n, words), dtype=torch.int32, device=dev)
    status = lib.abm_vpf_social_fields(
        _lib.fptr(xs), _lib.fptr(ys), _lib.fptr(ts), _lib.fptr(rs), float(radius),
        _lib.i32ptr(ex), _lib.i32ptr(pa), n, float(vision_range), 1 if visual_exclusion else 0,
        1 if patchwise else 0, int(rv), float(fov[0]), float(fov[1]), _lib.u32ptr(out),
        _lib.u64ptr(diag), ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    _lib.check(status, "abm_vpf_social_fields")
    if as_bits:
        return out
    words_np = out.cpu().numpy().view(np.uint32).astype("<u4").view(np.uint8)
    return np.unpackbits(words_np.reshape(n, -1), axis=1, bitorder="little")[:, : int(rv)]
