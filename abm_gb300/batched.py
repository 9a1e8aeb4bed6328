"""Batched parameter sweeps: many independent visual-flocking swarms in one launch per step.

The reference sweeps parameters by generating one .env file per combination and running one
simulation per file, sequentially or as separate processes
(abm/metarunner/metarunner.py:168-254, HPC_run_all_exp_distribute.sh).  ``BatchedSweep`` keeps
every instance's agents in one concatenated device state and advances all of them with one
``abm_vpf_flock_batched`` call per step (each agent only sees its own instance), with the step
loop captured in CUDA graphs of ``chunk`` steps.
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np
import torch

from . import _lib
from .params import VFParams


class BatchedSweep:
    """instances: sequence of dicts with x, y, theta (and optionally v, alp0, bet0, v0,
    radius): one dict per independent swarm.  All instances share `params` (Rv, arena,
    boundary, GAM, ALP1, BET1, ...); ALP0 / BET0 / V0 / radius may differ per instance."""

    def __init__(self, params: VFParams, instances: Sequence[dict], device="cuda"):
        self.lib = _lib.load()
        self.params = params
        self.device = torch.device(device)
        sizes = np.array([len(inst["x"]) for inst in instances], np.int64)
        if np.any(sizes <= 0):
            raise ValueError("every instance needs at least one agent")
        self.sizes = sizes
        self.offsets = np.concatenate([[0], np.cumsum(sizes)]).astype(np.int64)
        n = int(self.offsets[-1])
        self.n = n
        def cat(key, default):
            parts = []
            for inst in instances:
                val = inst.get(key)
                arr = np.asarray(default if val is None else val, np.float32)
                parts.append(np.full(len(inst["x"]), float(arr), np.float32) if arr.ndim == 0
                             else arr.reshape(-1))
            return np.concatenate(parts)

        host = {"x": cat("x", 0.0), "y": cat("y", 0.0), "theta": cat("theta", 0.0),
                "v": cat("v", 0.0)}
        dev = lambda a, dt=torch.float32: torch.as_tensor(np.ascontiguousarray(a), dtype=dt,
                                                          device=self.device)
        self._bufs = [{k: dev(v) for k, v in host.items()},
                      {k: torch.empty(n, dtype=torch.float32, device=self.device)
                       for k in host}]
        self._cur = 0
        ov = {}
        for key, default in (("alp0", params.alp0), ("bet0", params.bet0), ("v0", params.v0),
                             ("radius", params.radius)):
            if any(inst.get(key) is not None for inst in instances):
                ov[key] = dev(cat(key, default))
        self.ov_tensors = ov
        self._ov = _lib.AbmAgentOverrides(_lib.fptr(ov.get("radius")), _lib.fptr(ov.get("alp0")),
                                          _lib.fptr(ov.get("bet0")), _lib.fptr(ov.get("v0")))
        inst_of = np.repeat(np.arange(len(sizes)), sizes)
        self.seg_begin = dev(self.offsets[inst_of], torch.int32)
        self.seg_end = dev(self.offsets[inst_of + 1], torch.int32)
        # largest instances first: their agents carry the most pairs
        order = np.argsort(-sizes[inst_of], kind="stable").astype(np.int32)
        self.order = dev(order, torch.int32)
        self._cparams = params.to_c()
        self.words = int(_lib.check(self.lib.abm_vpf_words(int(params.rv))))
        self.vpf_bits = torch.zeros((n, self.words), dtype=torch.int32, device=self.device)
        self.terms = torch.zeros((n, 6), dtype=torch.float64, device=self.device)
        self.diag = torch.zeros(_lib.ABM_DIAG_COUNT, dtype=torch.int64, device=self.device)
        self._graph = None
        self._graph_chunk = 0
        self._stream = None
        self._pol = None
        self._rec = None

    # ------------------------------------------------------------------ ensemble statistic
    def track_polarisation(self, capacity: int):
        """Record each instance's polarisation (|sum (cos, sin)| / N, the reference's
        DataLoader.calculate_polarization) after every step, on the device, for up to
        `capacity` steps (abm_vpf_polarisation, captured with the step in graphs)."""
        k = len(self.sizes)
        self._pol = torch.full((k, int(capacity)), float("nan"), dtype=torch.float64,
                               device=self.device)
        self._pol_step = torch.zeros(k, dtype=torch.int32, device=self.device)
        self._pol_off = torch.as_tensor(self.offsets.astype(np.int32), device=self.device)
        self._graph = None   # re-capture with the statistic

    def polarisation(self) -> np.ndarray:
        """(n_instances, steps) polarisation series recorded so far."""
        steps = int(self._pol_step.max().item())
        return self._pol[:, : min(steps, self._pol.shape[1])].cpu().numpy()

    def _record_polarisation(self, state, stream):
        _lib.check(self.lib.abm_vpf_polarisation(
            _lib.fptr(state["theta"]), self.n, _lib.i32ptr(self._pol_off), len(self.sizes),
            _lib.dptr(self._pol), self._pol.shape[1], _lib.i32ptr(self._pol_step),
            ctypes.c_void_p(stream.cuda_stream)), "abm_vpf_polarisation")

    # ------------------------------------------------------------------ recording
    def record_steps(self, capacity: int, vpf: bool = False):
        """Record every instance's state after each following step on the device
        (abm_vpf_record over the concatenated state, captured with the step in graphs), as the
        reference's RAM recorder does in each instance's own run (vf_sims.py:328-331), for up
        to `capacity` steps; vpf: also each step's VPF."""
        from .swarm import VfRecorder
        self._rec = VfRecorder(self.lib, self.n, self.words, capacity, vpf, self.device)
        self._graph = None   # re-capture with the recorder

    def instance_recording(self, k: int) -> dict:
        """Instance k's recorded series (posx, posy, orientation, velocity, optional vpf_bits:
        agents x steps) and the number of steps."""
        if self._rec is None:
            raise RuntimeError("no recording: call record_steps first")
        out = self._rec.series(int(self.offsets[k]), int(self.offsets[k + 1]))
        out["steps"] = self._rec.steps()
        return out

    def save_reference_run(self, k: int, folder: str, as_zarr: bool = False, env=None,
                           save_extracted_vfield: bool = False):
        """Write instance k's recording as the reference writes one simulation's data (JSON,
        or the zarr arrays of USE_ZARR_FORMAT=1, and env_params.json when `env` is given)."""
        from .recording import save_vf_run
        save_vf_run(folder, self.instance_recording(k), self.params.rv, as_zarr, env,
                    save_extracted_vfield)

    @staticmethod
    def _state(d):
        return _lib.AbmSwarmState(_lib.fptr(d["x"]), _lib.fptr(d["y"]), _lib.fptr(d["theta"]),
                                  _lib.fptr(d["v"]))

    def _launch(self, src: int, stream, want_vpf=False, want_terms=False) -> int:
        want_vpf = want_vpf or (self._rec is not None and self._rec.vpf_bits is not None)
        st_in = self._state(self._bufs[src])
        st_out = self._state(self._bufs[1 - src])
        status = self.lib.abm_vpf_flock_batched(
            ctypes.byref(st_in), ctypes.byref(st_out), self.n, _lib.i32ptr(self.seg_begin),
            _lib.i32ptr(self.seg_end), _lib.i32ptr(self.order), ctypes.byref(self._cparams),
            ctypes.byref(self._ov), _lib.u32ptr(self.vpf_bits) if want_vpf else None,
            _lib.dptr(self.terms) if want_terms else None, _lib.u64ptr(self.diag),
            ctypes.c_void_p(stream.cuda_stream))
        st = _lib.check(status, "abm_vpf_flock_batched")
        if self._pol is not None:
            self._record_polarisation(self._bufs[1 - src], stream)
        if self._rec is not None:
            self._rec.launch(self._state(self._bufs[1 - src]), self.vpf_bits, self.params.rv,
                             stream)
        return st

    def step(self, want_vpf=False, want_terms=False, stream=None) -> int:
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        st = self._launch(self._cur, s, want_vpf, want_terms)
        self._cur = 1 - self._cur
        return st

    def capture(self, chunk: int = 100):
        """Capture `chunk` steps (an even number, so the state ends in the buffer it started
        from) as a CUDA graph on a private stream, after warm-up launches on that stream."""
        if chunk <= 0 or chunk % 2:
            raise ValueError("chunk must be a positive even number")
        self._stream = torch.cuda.Stream(self.device)
        saved = {k: t.clone() for k, t in self._bufs[self._cur].items()}
        saved_pol = None if self._pol is None else (self._pol.clone(), self._pol_step.clone())
        saved_rec = None if self._rec is None else self._rec.step.clone()
        # the warm-up steps overwrite the state: they start once the copies are taken
        self._stream.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(self._stream):
            for _ in range(2):     # builds tables / workspace outside the capture
                self.step(stream=self._stream)
        self._stream.synchronize()
        for k, t in saved.items():
            self._bufs[self._cur][k].copy_(t)
        if saved_pol is not None:   # the warm-up steps are not part of the run
            self._pol.copy_(saved_pol[0])
            self._pol_step.copy_(saved_pol[1])
        if saved_rec is not None:   # their records are overwritten by the run's
            self._rec.step.copy_(saved_rec)
        self._stream.wait_stream(torch.cuda.current_stream(self.device))
        g = torch.cuda.CUDAGraph()
        start = self._cur
        with torch.cuda.graph(g, stream=self._stream):
            for k in range(chunk):
                self._launch((start + k) % 2, self._stream)
        self._graph, self._graph_chunk, self._graph_start = g, chunk, start
        torch.cuda.current_stream(self.device).wait_stream(self._stream)

    def run(self, steps: int, chunk: int = 100):
        """Advance `steps` steps with graph replays of `chunk` steps (plus single steps)."""
        if self._graph is None or self._graph_chunk != chunk:
            self.capture(chunk)
        if self._cur != self._graph_start:
            self.step()
            steps -= 1
        while steps >= chunk:
            self._graph.replay()
            steps -= chunk
        for _ in range(steps):
            self.step()

    # ------------------------------------------------------------------ access
    def state_numpy(self) -> dict:
        return {k: t.cpu().numpy() for k, t in self._bufs[self._cur].items()}

    def instance_state(self, k: int) -> dict:
        a, b = int(self.offsets[k]), int(self.offsets[k + 1])
        return {key: t[a:b].cpu().numpy() for key, t in self._bufs[self._cur].items()}

    def vpf_numpy(self) -> np.ndarray:
        words = self.vpf_bits.cpu().numpy().view(np.uint32).astype("<u4").view(np.uint8)
        bits = np.unpackbits(words.reshape(self.n, -1), axis=1, bitorder="little")
        return bits[:, : self.params.rv]


def sweep_instances(n_instances: int = 512, n_min: int = 10, n_max: int = 500,
                    alp_grid=(16, 32), alp_range=(0.1, 3.0), width=1000.0, height=1000.0,
                    pad=30.0, radius=10.0, seed: int = 3):
    """Seeded instances of the batched-sweep workload: N_i uniform in [n_min, n_max], (ALP0,
    BET0) on an alp_grid[0] x alp_grid[1] grid over alp_range, positions uniform in the arena,
    headings uniform, speeds 0."""
    rng = np.random.default_rng(seed)
    a0 = np.linspace(alp_range[0], alp_range[1], alp_grid[0])
    b0 = np.linspace(alp_range[0], alp_range[1], alp_grid[1])
    out = []
    for k in range(n_instances):
        n = int(rng.integers(n_min, n_max + 1))
        out.append({"x": rng.uniform(pad - radius, pad + width - radius, n).astype(np.float32),
                    "y": rng.uniform(pad - radius, pad + height - radius, n).astype(np.float32),
                    "theta": rng.uniform(0, 2 * np.pi, n).astype(np.float32),
                    "v": np.zeros(n, np.float32),
                    "alp0": float(a0[(k // alp_grid[1]) % alp_grid[0]]),
                    "bet0": float(b0[k % alp_grid[1]])})
    return out
