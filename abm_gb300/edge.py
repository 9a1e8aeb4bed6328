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


class _Stepper:
    """One rollout's forward launches with their ctypes arguments built once: parameters,
    stream, and the state structs of the buffers it steps between."""

    def __init__(self, lib, base, pv, dtype, use_asin, stream):
        self.fwd, self.bwd, _ = _fns(lib, dtype)
        self.cp = _cparams(base, pv)
        self.asin = 1 if use_asin else 0
        self.stream = ctypes.c_void_p(stream.cuda_stream)
        self._structs = {}

    def struct(self, bufs):
        key = tuple(t.data_ptr() for t in bufs)
        st = self._structs.get(key)
        if st is None:
            st = self._structs[key] = _state(bufs)
        return st

    def step(self, cur, nxt):
        _lib.check(self.fwd(ctypes.byref(self.struct(cur)), ctypes.byref(self.struct(nxt)),
                            cur[0].numel(), ctypes.byref(self.cp), self.asin, None, self.stream),
                   "abm_vpf_edge_fwd")


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
        stepper = _Stepper(lib, base, pv, dtype, use_asin, stream)
        ckpts = []
        for k in range(steps):
            if k % checkpoint == 0:
                ckpts.append([t.clone() for t in cur])
            stepper.step(cur, nxt)
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
        # gradient buffers as rows of (4, n) arrays: the adjoint clears one in a single memset
        G = torch.zeros((4, n), dtype=dtype, device=dev)
        for r, t in enumerate((gx, gy, gth, gv)):
            if t is not None:
                G[r].copy_(t)
        Gin = torch.empty_like(G)
        g, gin = list(G.unbind(0)), list(Gin.unbind(0))
        gparams = torch.zeros(5, dtype=torch.float64, device=dev)
        stepper = _Stepper(lib, base, pv, dtype, use_asin, stream)
        gp_ptr = _lib.dptr(gparams)
        # the states of one segment: the checkpoint, then K - 1 recomputed ones (reused)
        seg_bufs = [[torch.empty_like(t) for t in ctx.ckpts[0]] for _ in range(K - 1)]
        for seg in range(len(ctx.ckpts) - 1, -1, -1):
            t0 = seg * K
            t1 = min(t0 + K, steps)
            states = [ctx.ckpts[seg]] + seg_bufs[:t1 - t0 - 1]
            for k in range(t1 - t0 - 1):   # recompute the segment from its checkpoint
                stepper.step(states[k], states[k + 1])
            for k in range(t1 - 1, t0 - 1, -1):
                _lib.check(bwd(
                    ctypes.byref(stepper.struct(states[k - t0])),
                    ctypes.byref(stepper.struct(g)), ctypes.byref(stepper.struct(gin)),
                    gp_ptr, n, ctypes.byref(stepper.cp), stepper.asin, stepper.stream),
                    "abm_vpf_edge_bwd")
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
