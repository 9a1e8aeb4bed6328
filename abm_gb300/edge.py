"""Differentiable visual flocking: the continuum edge form with a hand-written adjoint.

``rollout(params, x0, y0, theta0, v0, steps)`` advances a swarm ``steps`` steps with the edge
form of the VSWRM integrals (abm_vpf_edge_fwd) and is a ``torch.autograd.Function``: its
backward runs the adjoint kernel (abm_vpf_edge_bwd) step by step in reverse, recomputing each
segment of ``checkpoint`` steps from a stored checkpoint, and returns gradients with respect to
the parameter vector (alp0, alp1, bet0, bet1, v0) and the initial state.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math

import torch

from . import _lib
from .params import VFParams

PARAM_NAMES = ("alp0", "alp1", "bet0", "bet1", "v0")


def _state(d):
    if d[0].dtype == torch.float64:
        return _lib.AbmSwarmStateF64(*[_lib.dptr(t) for t in d])
    return _lib.AbmSwarmState(*[_lib.fptr(t) for t in d])


def _fns(lib, dtype):
    if dtype == torch.float64:
        return lib.abm_vpf_edge_fwd_f64, lib.abm_vpf_edge_bwd_f64, _lib.dptr
    return lib.abm_vpf_edge_fwd, lib.abm_vpf_edge_bwd, _lib.fptr


def _cparams(base: VFParams, pvec) -> _lib.AbmVfParams:
    vals = dict(zip(PARAM_NAMES, (float(v) for v in pvec)))
    return dataclasses.replace(base, **vals).to_c()


def edge_step(lib, base, pvec, cur, nxt, use_asin, stream, terms=None):
    cp = _cparams(base, pvec)
    fwd, _, ptr = _fns(lib, cur[0].dtype)
    _lib.check(fwd(ctypes.byref(_state(cur)), ctypes.byref(_state(nxt)), cur[0].numel(),
                   ctypes.byref(cp), 1 if use_asin else 0, ptr(terms),
                   ctypes.c_void_p(stream.cuda_stream)), "abm_vpf_edge_fwd")


class _EdgeRollout(torch.autograd.Function):
    @staticmethod
    def forward(ctx, pvec, x0, y0, th0, v0, base, steps, checkpoint, use_asin):
        lib = _lib.load()
        dev = x0.device
        stream = torch.cuda.current_stream(dev)
        pv = [float(v) for v in pvec.detach().cpu().tolist()]
        dtype = torch.float64 if x0.dtype == torch.float64 else torch.float32
        cur = [t.detach().to(dtype).contiguous().clone() for t in (x0, y0, th0, v0)]
        nxt = [torch.empty_like(t) for t in cur]
        ckpts = []
        for k in range(steps):
            if k % checkpoint == 0:
                ckpts.append([t.clone() for t in cur])
            edge_step(lib, base, pv, cur, nxt, use_asin, stream)
            cur, nxt = nxt, cur
        ctx.base, ctx.steps, ctx.checkpoint, ctx.use_asin = base, steps, checkpoint, use_asin
        ctx.pv = pv
        ctx.ckpts = ckpts
        ctx.pdtype = pvec.dtype
        return tuple(t.clone() for t in cur)

    @staticmethod
    def backward(ctx, gx, gy, gth, gv):
        lib = _lib.load()
        base, steps, K, use_asin, pv = ctx.base, ctx.steps, ctx.checkpoint, ctx.use_asin, ctx.pv
        dev = ctx.ckpts[0][0].device
        dtype = ctx.ckpts[0][0].dtype
        _, bwd, _ = _fns(lib, dtype)
        stream = torch.cuda.current_stream(dev)
        n = ctx.ckpts[0][0].numel()
        zeros = lambda t: torch.zeros(n, dtype=dtype, device=dev) if t is None else t
        g = [zeros(t).to(dtype).contiguous() for t in (gx, gy, gth, gv)]
        gin = [torch.empty_like(t) for t in g]
        gparams = torch.zeros(5, dtype=torch.float64, device=dev)
        cp = _cparams(base, pv)
        for seg in range(len(ctx.ckpts) - 1, -1, -1):
            t0 = seg * K
            t1 = min(t0 + K, steps)
            # recompute the segment's states from its checkpoint
            states = [ctx.ckpts[seg]]
            cur = [t.clone() for t in ctx.ckpts[seg]]
            for _ in range(t0, t1 - 1):
                nxt = [torch.empty_like(t) for t in cur]
                edge_step(lib, base, pv, cur, nxt, use_asin, stream)
                states.append(nxt)
                cur = nxt
            for k in range(t1 - 1, t0 - 1, -1):
                st = states[k - t0]
                _lib.check(bwd(
                    ctypes.byref(_state(st)), ctypes.byref(_state(g)), ctypes.byref(_state(gin)),
                    _lib.dptr(gparams), n, ctypes.byref(cp), 1 if use_asin else 0,
                    ctypes.c_void_p(stream.cuda_stream)), "abm_vpf_edge_bwd")
                g, gin = gin, g
        gp = gparams.to(ctx.pdtype)
        return (gp, g[0].clone(), g[1].clone(), g[2].clone(), g[3].clone(), None, None, None,
                None)


def rollout(pvec, x0, y0, theta0, v0, base: VFParams, steps: int, checkpoint: int = 20,
            use_asin: bool = False):
    """Final state (x, y, theta, v) after `steps` edge-form steps; differentiable w.r.t.
    pvec = (alp0, alp1, bet0, bet1, v0) and the initial state.  float32 inputs run the float32
    kernels, float64 inputs the double-precision ones (needed when gradients must follow an FP64
    reference through the arc merge / split events of long horizons)."""
    return _EdgeRollout.apply(pvec, x0, y0, theta0, v0, base, steps, checkpoint, use_asin)


def flocking_loss(x, y, theta, target, radius=0.0):
    """1 - polarisation (data_loader.py:1818-1824) + mean squared error of the mean centre
    position to `target` (the differentiable workload's trajectory loss)."""
    n = theta.numel()
    pol = torch.sqrt(torch.cos(theta).sum() ** 2 + torch.sin(theta).sum() ** 2) / n
    mx, my = (x + radius).mean(), (y + radius).mean()
    return 1.0 - pol + ((mx - target[0]) ** 2 + (my - target[1]) ** 2) / 2.0


def edge_terms(state, base: VFParams, pvec=None, use_asin=False):
    """(n, 4) integrals {blob_c, blob_s, edge_c, edge_s} of the edge form for one state."""
    lib = _lib.load()
    dtype = torch.float64 if state[0].dtype == torch.float64 else torch.float32
    cur = [t.to(dtype).contiguous() for t in state]
    nxt = [torch.empty_like(t) for t in cur]
    terms = torch.empty((cur[0].numel(), 4), dtype=dtype, device=cur[0].device)
    pv = [getattr(base, k) for k in PARAM_NAMES] if pvec is None else pvec
    edge_step(lib, base, pv, cur, nxt, use_asin, torch.cuda.current_stream(cur[0].device), terms)
    return terms
