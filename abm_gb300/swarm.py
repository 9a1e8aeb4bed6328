"""Device-resident visual-flocking swarm: the batched replacement of the reference step loop.

``VFSimulation.step_sim`` (abm/projects/visual_flocking/vf_simulation/vf_sims.py:291-340)
calls ``VFAgent.update`` for every agent in pygame group order; each update computes the
agent's VPF (``calc_soc_v_proj``, vf_agent.py:216-237), the VSWRM increments
(``perform_action``, :263-287), moves the agent (:289-309) and applies the boundary rule
(agent.py:347-394 / vf_agent.py:188-204).  ``VFSwarm.step`` does all agents in one kernel
launch from a snapshot of the state (Jacobi order), on torch-owned device memory.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np
import torch

from . import _lib
from .params import VFParams


def _dev_tensor(a, device, dtype=torch.float32):
    if a is None:
        return None
    t = torch.as_tensor(np.asarray(a) if not torch.is_tensor(a) else a)
    return t.to(device=device, dtype=dtype).contiguous()


class VfRecorder:
    """Device series of abm_vpf_record: n agents, `capacity` steps, optionally the VPF."""

    def __init__(self, lib, n: int, words: int, capacity: int, vpf: bool, device):
        cap = int(capacity)
        self.lib, self.n, self.words, self.capacity = lib, n, words, cap
        self.step = torch.zeros(2, dtype=torch.int32, device=device)
        self.posx = torch.zeros((n, cap), dtype=torch.int32, device=device)
        self.posy = torch.zeros((n, cap), dtype=torch.int32, device=device)
        self.orientation = torch.zeros((n, cap), dtype=torch.float32, device=device)
        self.velocity = torch.zeros((n, cap), dtype=torch.float32, device=device)
        self.vpf_bits = (torch.zeros((n, cap, words), dtype=torch.int32, device=device)
                         if vpf else None)
        self.struct = _lib.AbmVfRecording(
            cap, _lib.i32ptr(self.step), _lib.i32ptr(self.posx), _lib.i32ptr(self.posy),
            _lib.fptr(self.orientation), _lib.fptr(self.velocity), _lib.u32ptr(self.vpf_bits))

    def launch(self, state: "_lib.AbmSwarmState", vpf_bits, rv: int, stream):
        _lib.check(self.lib.abm_vpf_record(
            ctypes.byref(state), self.n,
            _lib.u32ptr(vpf_bits) if self.vpf_bits is not None else None, int(rv),
            ctypes.byref(self.struct), ctypes.c_void_p(stream.cuda_stream)), "abm_vpf_record")

    def steps(self) -> int:
        return min(int(self.step[0].item()), self.capacity)

    def series(self, a: int = 0, b: Optional[int] = None) -> dict:
        """Rows a:b of the recorded steps as numpy: posx, posy, orientation, velocity (rows,
        steps) and vpf_bits (rows, steps, words) uint32 when recorded."""
        t = self.steps()
        out = {k: getattr(self, k)[a:b, :t].cpu().numpy()
               for k in ("posx", "posy", "orientation", "velocity")}
        if self.vpf_bits is not None:
            out["vpf_bits"] = self.vpf_bits[a:b, :t].cpu().numpy().view(np.uint32)
        return out


class VFSwarm:
    """N visual-flocking agents of one arena, state in float32 on `device`.

    x, y: top-left positions (the reference's ``agent.position``); theta: orientation in
    [0, 2pi]; v: speed (the reference starts at 0).  radius / alp0 / bet0 / v0: optional
    per-agent overrides (object_sizes and VFAgent.ALP0/BET0/V0)."""

    def __init__(self, params: VFParams, x, y, theta, v=None, radius=None, alp0=None,
                 bet0=None, v0=None, device="cuda"):
        self.lib = _lib.load()
        self.params = params
        self.device = torch.device(device)
        n = len(x)
        self.n = n
        self._cur = {k: _dev_tensor(a, self.device) for k, a in
                     (("x", x), ("y", y), ("theta", theta),
                      ("v", np.zeros(n, np.float32) if v is None else v))}
        self._nxt = {k: torch.empty_like(t) for k, t in self._cur.items()}
        self.radius = _dev_tensor(radius, self.device)
        self.alp0 = _dev_tensor(alp0, self.device)
        self.bet0 = _dev_tensor(bet0, self.device)
        self.v0 = _dev_tensor(v0, self.device)
        self.words = int(_lib.check(self.lib.abm_vpf_words(int(params.rv)), "abm_vpf_words"))
        self.vpf_bits = torch.zeros((n, self.words), dtype=torch.int32, device=self.device)
        self.terms = torch.zeros((n, 6), dtype=torch.float64, device=self.device)
        self.diag = torch.zeros(_lib.ABM_DIAG_COUNT, dtype=torch.int64, device=self.device)
        self._cparams = params.to_c()
        self._ov = _lib.AbmAgentOverrides(_lib.fptr(self.radius), _lib.fptr(self.alp0),
                                          _lib.fptr(self.bet0), _lib.fptr(self.v0))
        self.last_status = 0

    @staticmethod
    def _state_struct(d):
        return _lib.AbmSwarmState(_lib.fptr(d["x"]), _lib.fptr(d["y"]), _lib.fptr(d["theta"]),
                                  _lib.fptr(d["v"]))

    def step(self, want_vpf: bool = False, want_terms: bool = False,
             stream: Optional[torch.cuda.Stream] = None) -> int:
        """Advance every agent by one timestep (one kernel launch, asynchronous)."""
        rec = getattr(self, "_rec", None)
        want_vpf = want_vpf or (rec is not None and rec.vpf_bits is not None)
        st_in = self._state_struct(self._cur)
        st_out = self._state_struct(self._nxt)
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        status = self.lib.abm_vpf_flock_step(
            ctypes.byref(st_in), ctypes.byref(st_out), self.n, ctypes.byref(self._cparams),
            ctypes.byref(self._ov), _lib.u32ptr(self.vpf_bits) if want_vpf else None,
            _lib.dptr(self.terms) if want_terms else None, _lib.u64ptr(self.diag),
            ctypes.c_void_p(s.cuda_stream))
        self.last_status = _lib.check(status, "abm_vpf_flock_step")
        self._cur, self._nxt = self._nxt, self._cur
        if getattr(self, "_pol", None) is not None:
            _lib.check(self.lib.abm_vpf_polarisation(
                _lib.fptr(self._cur["theta"]), self.n, None, 1, _lib.dptr(self._pol),
                self._pol.shape[1], _lib.i32ptr(self._pol_step),
                ctypes.c_void_p(s.cuda_stream)), "abm_vpf_polarisation")
        if rec is not None:
            rec.launch(self._state_struct(self._cur), self.vpf_bits, self.params.rv, s)
        return self.last_status

    def record_steps(self, capacity: int, vpf: bool = False):
        """Record the state after every following step on the device (abm_vpf_record), as the
        reference's RAM recorder does each step (vf_sims.py:328-331), for up to `capacity`
        steps; vpf: also the step's VPF (its edges go into the reference's files)."""
        self._rec = VfRecorder(self.lib, self.n, self.words, capacity, vpf, self.device)

    def recording(self) -> dict:
        """The recorded series on the host (see VfRecorder.series) and the number of steps."""
        if getattr(self, "_rec", None) is None:
            raise RuntimeError("no recording: call record_steps first")
        out = self._rec.series()
        out["steps"] = self._rec.steps()
        return out

    def save_reference_run(self, folder: str, as_zarr: bool = False, env=None,
                           save_extracted_vfield: bool = False):
        """Write the recording in the reference's layout: agent_data.json / resource_data.json,
        or the ag_*.zarr arrays (USE_ZARR_FORMAT=1), plus env_params.json when `env` is given
        (the end of VFSimulation.start, vf_sims.py:373-381)."""
        from .recording import save_vf_run
        save_vf_run(folder, self.recording(), self.params.rv, as_zarr, env,
                    save_extracted_vfield)

    def track_polarisation(self, capacity: int):
        """Record the swarm's polarisation (|sum (cos, sin)| / N, the reference's
        DataLoader.calculate_polarization) after every step, on the device."""
        self._pol = torch.full((1, int(capacity)), float("nan"), dtype=torch.float64,
                               device=self.device)
        self._pol_step = torch.zeros(1, dtype=torch.int32, device=self.device)

    def polarisation(self) -> np.ndarray:
        steps = int(self._pol_step.item())
        return self._pol[0, : min(steps, self._pol.shape[1])].cpu().numpy()

    def run(self, steps: int, stream=None, graph_chunk: int = 0) -> int:
        """Advance `steps` steps.  graph_chunk >= 2: one library call (abm_vpf_flock_run, or
        abm_vpf_flock_run_recorded when recording) that replays a CUDA graph of graph_chunk
        steps (not with polarisation tracking); the stream must then be a non-default one.
        Otherwise one abm_vpf_flock_step call per step."""
        rec = getattr(self, "_rec", None)
        if graph_chunk < 2 or getattr(self, "_pol", None) is not None:
            st = 0
            for _ in range(steps):
                st = self.step(stream=stream)
            return st
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        if rec is not None:   # step + record in the library's graph
            status = self.lib.abm_vpf_flock_run_recorded(
                ctypes.byref(self._state_struct(self._cur)),
                ctypes.byref(self._state_struct(self._nxt)), self.n, ctypes.byref(self._cparams),
                ctypes.byref(self._ov), int(steps), int(graph_chunk),
                _lib.u32ptr(self.vpf_bits) if rec.vpf_bits is not None else None,
                ctypes.byref(rec.struct), _lib.u64ptr(self.diag), ctypes.c_void_p(s.cuda_stream))
            self.last_status = _lib.check(status, "abm_vpf_flock_run_recorded")
            if steps % 2:
                self._cur, self._nxt = self._nxt, self._cur
            return self.last_status
        status = self.lib.abm_vpf_flock_run(
            ctypes.byref(self._state_struct(self._cur)), ctypes.byref(self._state_struct(self._nxt)),
            self.n, ctypes.byref(self._cparams), ctypes.byref(self._ov), int(steps),
            int(graph_chunk), _lib.u64ptr(self.diag), ctypes.c_void_p(s.cuda_stream))
        self.last_status = _lib.check(status, "abm_vpf_flock_run")
        if steps % 2:
            self._cur, self._nxt = self._nxt, self._cur
        return self.last_status

    # ------------------------------------------------------------------ state access
    @property
    def state(self) -> dict:
        """Current state as float32 device tensors (x, y, theta, v)."""
        return self._cur

    def state_numpy(self) -> dict:
        return {k: t.detach().cpu().numpy() for k, t in self._cur.items()}

    def set_state(self, x, y, theta, v):
        for k, a in (("x", x), ("y", y), ("theta", theta), ("v", v)):
            self._cur[k].copy_(torch.as_tensor(np.asarray(a), dtype=torch.float32))

    def vpf_numpy(self) -> np.ndarray:
        """(n, Rv) uint8 VPF of the last step with want_vpf=True, raw pixel order."""
        words = self.vpf_bits.cpu().numpy().view(np.uint32).astype("<u4").view(np.uint8)
        bits = np.unpackbits(words.reshape(self.n, -1), axis=1, bitorder="little")
        return bits[:, : self.params.rv]

    def check_status(self, stream=None) -> None:
        """Synchronise the stream and raise AbmError(ABM_ERR_TIMEOUT) if a step kernel on this
        device gave up a bounded wait since the last check (abm_vpf_status; clears the flag)."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        _lib.check(_lib.load().abm_vpf_status(1, ctypes.c_void_p(s.cuda_stream)),
                   "abm_vpf_status")

    def diagnostics(self) -> dict:
        d = self.diag.cpu().numpy()
        return {"pairs_resolved": int(d[_lib.DIAG_PAIRS_RESOLVED]),
                "near_boundary": int(d[_lib.DIAG_NEAR_BOUNDARY]),
                "nonfinite": int(d[_lib.DIAG_NONFINITE]),
                "timeouts": int(d[_lib.DIAG_TIMEOUTS])}

    # ------------------------------------------------------------------ reference interop
    @classmethod
    def from_reference_agents(cls, agents, params: VFParams, device="cuda"):
        """Build from a list of reference VFAgent objects (pygame group order)."""
        ags = list(agents)
        x = np.array([a.position[0] for a in ags], np.float32)
        y = np.array([a.position[1] for a in ags], np.float32)
        th = np.array([a.orientation for a in ags], np.float32)
        v = np.array([a.velocity for a in ags], np.float32)
        r = np.array([a.radius for a in ags], np.float32)
        hetero = bool(np.any(r != r[0]))
        ov = {}
        for name in ("ALP0", "BET0", "V0"):
            vals = [getattr(a, name, None) for a in ags]
            if any(val is not None for val in vals):
                dflt = getattr(params, name.lower())
                ov[name.lower()] = np.array([dflt if val is None else val for val in vals],
                                            np.float32)
        return cls(params, x, y, th, v, radius=r if hetero else None, device=device, **ov)

    def write_back(self, agents):
        """Copy the current state into reference agent objects."""
        st = self.state_numpy()
        for i, a in enumerate(agents):
            a.position = [float(st["x"][i]), float(st["y"][i])]
            a.orientation = float(st["theta"][i])
            a.velocity = float(st["v"][i])


def step_host(lib, params_c, n, host_in, host_out, stream, overrides=None):
    """One step on HOST buffers through abm_vpf_flock_step_host (the drop-in call a per-step
    host loop makes): the library moves the state to the device and the result back, on
    `stream`.  host_* are dicts of float32 CPU tensors (page-locked for the fast path)."""
    st_in = VFSwarm._state_struct(host_in)
    st_out = VFSwarm._state_struct(host_out)
    status = lib.abm_vpf_flock_step_host(
        ctypes.byref(st_in), ctypes.byref(st_out), n, ctypes.byref(params_c),
        ctypes.byref(overrides) if overrides is not None else None,
        ctypes.c_void_p(stream.cuda_stream))
    _lib.check(status, "abm_vpf_flock_step_host")
    return status
