"""Collective foraging on the GPU: the reference's foraging simulation step (abm_forage_step).

``ForagingSim`` holds one arena (agents and resource patches) on the device and advances it
with ``abm_forage_step`` — agent-resource interaction (abm/simulation/sims.py:789-858), the
social visual projection field (Agent.calc_social_V_proj, abm/agent/agent.py:396-419) and the
agent update (Agent.update, agent.py:213-283) — optionally replaying CUDA graphs of 100 steps.
Agents start like Simulation.create_agents (sims.py:526-537: integer positions uniform over
the arena including a border overlap of one radius, orientation uniform) and patches like
create_resources / add_new_resource_patch (sims.py:332-374: integer positions without patch
overlap); the initial placement uses numpy's generator with the given seed, the step's own
draws come from the device generator with the same seed.

``efficiency`` is the reference's foraging efficiency (data_loader.py:1333-1346): units
collected per agent between two times divided by the elapsed time.
"""
from __future__ import annotations

import ctypes
import dataclasses
import math
from typing import Optional

import numpy as np
import torch

from . import _lib
from .recording import agents_dict, reference_json, resources_dict, save_reference_zarr

MODES = {0: "explore", 1: "relocate", 2: "exploit", 3: "pool", 4: "collide"}


@dataclasses.dataclass
class ForageParams:
    # decision processes (abm/contrib/decision_params.py defaults)
    T_w: float = 0.5
    Eps_w: float = 3.0
    g_w: float = 0.085
    B_w: float = 0.0
    w_max: float = 1.0
    T_u: float = 0.5
    Eps_u: float = 3.0
    g_u: float = 0.085
    B_u: float = 0.0
    u_max: float = 1.0
    S_wu: float = 0.25
    S_uw: float = 0.01
    F_N: float = 2.0
    F_R: float = 1.0
    Tau: int = 10
    # movement (abm/contrib/movement_params.py defaults)
    exp_vel_max: float = 1.0
    exp_theta_min: float = -0.3
    exp_theta_max: float = 0.3
    reloc_theta_max: float = 0.5
    exp_stop_ratio: float = 0.08
    # arena, agents, patches (the foraging workload)
    width: float = 1000.0
    height: float = 1000.0
    window_pad: float = 30.0
    agent_radius: float = 10.0
    consumption: float = 1.0
    pooling_time: int = 0
    teleport_exploit: bool = True
    regenerate_patches: bool = True
    allow_border_patch_overlap: bool = False
    min_resc_units: int = 1000
    max_resc_units: int = 1000
    min_resc_quality: float = 1.0
    max_resc_quality: float = 1.0
    patch_radius: float = 30.0
    # social channel
    rv: int = 1200
    fov: float = 1.0                  # AGENT_FOV: field of view (-fov pi, fov pi)
    vision_range: float = 2000.0
    visual_exclusion: bool = True
    patchwise_exclusion: bool = True
    seed: int = 0
    # agent-agent collisions (AGENT_AGENT_COLLISION, GHOST_WHILE_EXPLOIT of the root .env)
    collide_agents: bool = False
    ghost_mode: bool = True

    _FP = ("T_w", "Eps_w", "g_w", "B_w", "w_max", "T_u", "Eps_u", "g_u", "B_u", "u_max", "S_wu",
           "S_uw", "F_N", "F_R", "exp_vel_max", "exp_theta_min", "exp_theta_max",
           "reloc_theta_max", "exp_stop_ratio", "width", "height", "window_pad", "agent_radius",
           "consumption", "min_resc_quality", "max_resc_quality", "patch_radius")
    _IP = ("Tau", "pooling_time", "teleport_exploit", "regenerate_patches",
           "allow_border_patch_overlap", "min_resc_units", "max_resc_units", "rv",
           "visual_exclusion", "patchwise_exclusion", "collide_agents", "ghost_mode")

    def to_c(self) -> "_lib.AbmForageParams":
        c = _lib.AbmForageParams()
        for k in self._FP:
            setattr(c, k, float(getattr(self, k)))
        for k in self._IP:
            setattr(c, k, int(getattr(self, k)))
        c.fov0, c.fov1 = -self.fov * math.pi, self.fov * math.pi
        c.vision_range = float(self.vision_range)
        c.seed = int(self.seed) & 0xFFFFFFFFFFFFFFFF
        return c

    def oracle_arrays(self):
        """(FP[30], IP[12], seed) in the layout of the oracle's orc_forage_step."""
        fp = [float(getattr(self, k)) for k in self._FP]
        fp += [-self.fov * math.pi, self.fov * math.pi, float(self.vision_range)]
        ip = [int(getattr(self, k)) for k in self._IP]
        return np.array(fp, np.float64), np.array(ip, np.int32), int(self.seed)

    @classmethod
    def from_arrays(cls, fp, ip, seed: int = 0) -> "ForageParams":
        """Inverse of oracle_arrays() (arrays without the two collision switches leave
        collisions off)."""
        kw = {k: float(fp[j]) for j, k in enumerate(cls._FP)}
        kw.update({k: int(ip[j]) for j, k in enumerate(cls._IP) if j < len(ip)})
        for k in ("teleport_exploit", "regenerate_patches", "allow_border_patch_overlap",
                  "visual_exclusion", "patchwise_exclusion", "collide_agents", "ghost_mode"):
            if k not in kw:
                continue
            kw[k] = bool(kw[k])
        fov0, fov1, vr = (float(v) for v in fp[len(cls._FP):len(cls._FP) + 3])
        return cls(**kw, fov=fov1 / math.pi, vision_range=vr, seed=int(seed))

    @classmethod
    def from_env(cls, env: dict, **over) -> "ForageParams":
        """From a reference .env mapping (abm/app.py:27-62, decision_params.py,
        movement_params.py); keys that are absent keep the defaults."""
        f = lambda key, d: float(env.get(key, d))
        i = lambda key, d: int(float(env.get(key, d)))
        d = cls()
        p = cls(T_w=f("DEC_TW", d.T_w), Eps_w=f("DEC_EPSW", d.Eps_w), g_w=f("DEC_GW", d.g_w),
                B_w=f("DEC_BW", d.B_w), w_max=f("DEC_WMAX", d.w_max), T_u=f("DEC_TU", d.T_u),
                Eps_u=f("DEC_EPSU", d.Eps_u), g_u=f("DEC_GU", d.g_u), B_u=f("DEC_BU", d.B_u),
                u_max=f("DEC_UMAX", d.u_max), S_wu=f("DEC_SWU", d.S_wu),
                S_uw=f("DEC_SUW", d.S_uw), Tau=i("DEC_TAU", d.Tau), F_N=f("DEC_FN", d.F_N),
                F_R=f("DEC_FR", d.F_R), exp_vel_max=f("MOV_EXP_VEL_MAX", d.exp_vel_max),
                exp_theta_min=f("MOV_EXP_TH_MIN", d.exp_theta_min),
                exp_theta_max=f("MOV_EXP_TH_MAX", d.exp_theta_max),
                reloc_theta_max=f("MOV_REL_TH_MAX", d.reloc_theta_max),
                exp_stop_ratio=f("CONS_STOP_RATIO", d.exp_stop_ratio),
                width=i("ENV_WIDTH", d.width), height=i("ENV_HEIGHT", d.height),
                agent_radius=i("RADIUS_AGENT", d.agent_radius),
                consumption=i("AGENT_CONSUMPTION", d.consumption),
                pooling_time=i("POOLING_TIME", d.pooling_time),
                teleport_exploit=bool(i("TELEPORT_TO_MIDDLE", d.teleport_exploit)),
                regenerate_patches=bool(i("REGENERATE_PATCHES", d.regenerate_patches)),
                allow_border_patch_overlap=bool(i("PATCH_BORDER_OVERLAP",
                                                  d.allow_border_patch_overlap)),
                min_resc_units=i("MIN_RESOURCE_PER_PATCH", d.min_resc_units),
                max_resc_units=i("MAX_RESOURCE_PER_PATCH", d.max_resc_units),
                min_resc_quality=f("MIN_RESOURCE_QUALITY", d.min_resc_quality),
                max_resc_quality=f("MAX_RESOURCE_QUALITY", d.max_resc_quality),
                patch_radius=i("RADIUS_RESOURCE", d.patch_radius),
                rv=i("VISUAL_FIELD_RESOLUTION", d.rv), fov=f("AGENT_FOV", d.fov),
                vision_range=i("VISION_RANGE", d.vision_range),
                visual_exclusion=bool(i("VISUAL_EXCLUSION", d.visual_exclusion)),
                patchwise_exclusion=bool(i("PATCHWISE_SOCIAL_EXCLUSION",
                                           d.patchwise_exclusion)),
                collide_agents=bool(i("AGENT_AGENT_COLLISION", d.collide_agents)),
                ghost_mode=bool(i("GHOST_WHILE_EXPLOIT", d.ghost_mode)))
        # sims.py:176-179: a negative maximum means a constant (units: randint(min, min + 1))
        if p.max_resc_quality < 0:
            p.max_resc_quality = p.min_resc_quality
        if p.max_resc_units < 0:
            p.max_resc_units = p.min_resc_units + 1
        return dataclasses.replace(p, **over)


AGENT_FIELDS = (("x", np.float32), ("y", np.float32), ("theta", np.float32), ("v", np.float32),
                ("w", np.float64), ("u", np.float64), ("collected", np.float64),
                ("collected_before", np.float64), ("mode", np.int32),
                ("override_mode", np.int32), ("env_status", np.int32),
                ("env_status_before", np.int32), ("pool_success", np.int32),
                ("patch_id", np.int32), ("novelty", np.uint32), ("draws", np.uint64),
                ("ipriv", np.float64))
PATCH_FIELDS = (("x", np.float64), ("y", np.float64), ("radius", np.float64),
                ("units", np.float64), ("left", np.float64), ("quality", np.float64),
                ("id", np.int32), ("draws", np.uint64))
_TORCH = {np.float32: torch.float32, np.float64: torch.float64, np.int32: torch.int32,
          np.uint32: torch.int32, np.uint64: torch.int64}


def initial_state(p: ForageParams, n_agents: int, n_patches: int, seed: int = 0):
    """(agents, patches) host dicts placed like Simulation.create_agents / create_resources
    (sims.py:526-542, 332-374), with numpy's generator seeded by `seed`."""
    rng = np.random.default_rng(seed)
    R, pad, W, H = p.agent_radius, p.window_pad, p.width, p.height
    agents = {k: np.zeros(n_agents, dt) for k, dt in AGENT_FIELDS}
    agents["x"][:] = rng.integers(int(pad - R), int(W + pad - R), n_agents)
    agents["y"][:] = rng.integers(int(pad - R), int(H + pad - R), n_agents)
    agents["theta"][:] = rng.uniform(0, 2 * np.pi, n_agents)
    agents["override_mode"][:] = -1
    agents["patch_id"][:] = -1
    patches = {k: np.zeros(n_patches, dt) for k, dt in PATCH_FIELDS}
    r = p.patch_radius
    for k in range(n_patches):
        for _ in range(10001):
            if p.allow_border_patch_overlap:
                x = rng.integers(int(pad - r), int(W + pad - r))
                y = rng.integers(int(pad - r), int(H + pad - r))
            else:
                x = rng.integers(int(pad), int(W + pad - 2 * r))
                y = rng.integers(int(pad), int(H + pad - 2 * r))
            clear = all((x - patches["x"][q]) ** 2 + (y - patches["y"][q]) ** 2 >= (2 * r) ** 2
                        for q in range(k))
            if clear:
                break
        else:
            raise RuntimeError("could not place the resource patches without overlap")
        units = (rng.integers(p.min_resc_units, p.max_resc_units)
                 if p.max_resc_units > p.min_resc_units else p.min_resc_units)
        patches["x"][k], patches["y"][k], patches["radius"][k] = x, y, r
        patches["units"][k] = patches["left"][k] = units
        patches["quality"][k] = rng.uniform(p.min_resc_quality, p.max_resc_quality)
        patches["id"][k] = k + 1
    return agents, patches


class ForagingSim:
    """One foraging arena on the GPU."""

    def __init__(self, params: ForageParams, n_agents: int = 100, n_patches: int = 3,
                 init_seed: int = 0, agents=None, patches=None, device="cuda",
                 record_steps: int = 0):
        self.lib = _lib.load()
        self.params = params
        self.device = torch.device(device)
        if agents is None or patches is None:
            agents, patches = initial_state(params, n_agents, n_patches, init_seed)
        self.n = len(agents["x"])
        self.np = len(patches["x"])
        n0 = len(agents["x"])
        self.ag = {k: self._dev(agents[k] if k in agents else np.zeros(n0, dt), dt)
                   for k, dt in AGENT_FIELDS}
        self.pt = {k: self._dev(patches[k], dt) for k, dt in PATCH_FIELDS}
        self.words = int(_lib.check(self.lib.abm_vpf_words(int(params.rv)), "abm_vpf_words"))
        self.soc_bits = torch.zeros((self.n, self.words), dtype=torch.int32, device=self.device)
        self.scratch = torch.zeros(2 * max(self.n, 1), dtype=torch.int32, device=self.device)
        self.diag = torch.zeros(_lib.ABM_DIAG_COUNT, dtype=torch.int64, device=self.device)
        self._cparams = params.to_c()
        self._agent_struct = _lib.AbmForagerState(
            *[ctypes.cast(self.ag[k].data_ptr(), ctype) for k, ctype in _lib.FORAGER_FIELDS])
        self._patch_struct = _lib.AbmPatchState(
            *[ctypes.cast(self.pt[k].data_ptr(), ctype) for k, ctype in _lib.PATCH_FIELDS])
        self.t = 0
        self._graph = None
        self.rec = None
        if record_steps > 0:
            self._init_recording(int(record_steps))

    # ------------------------------------------------------------------ recording
    _REC_AGENT = (("posx", torch.int32), ("posy", torch.int32), ("orientation", torch.float32),
                  ("velocity", torch.float32), ("w", torch.float64), ("u", torch.float64),
                  ("ipriv", torch.float64), ("collected", torch.float64),
                  ("mode", torch.int32), ("patch_id", torch.int32))
    _REC_PATCH = (("res_posx", torch.int32), ("res_posy", torch.int32),
                  ("res_left", torch.float64), ("res_quality", torch.float64),
                  ("res_id", torch.int32))

    def _init_recording(self, cap):
        d = self.device
        rec = {k: torch.zeros(self.n * cap, dtype=dt, device=d) for k, dt in self._REC_AGENT}
        rec.update({k: torch.zeros(max(self.np, 1) * cap, dtype=dt, device=d)
                    for k, dt in self._REC_PATCH})
        rec["soc_bits"] = torch.zeros(self.n * cap * self.words, dtype=torch.int32, device=d)
        rec["step"] = torch.zeros(1, dtype=torch.int32, device=d)
        self.rec, self.rec_capacity, self.rec_t0 = rec, cap, self.t
        self._rec_struct = _lib.AbmForageRecording(
            cap, ctypes.cast(rec["step"].data_ptr(), _lib.c_i32_p),
            *[ctypes.cast(rec[k].data_ptr(), c) for k, c in _lib.RECORDING_FIELDS])

    def recording(self) -> dict:
        """The recorded series on the host: agent fields (n, steps), patch fields
        (n_patches, steps), soc_bits (n, steps, words), and the number of steps."""
        if self.rec is None:
            raise RuntimeError("this simulation was created without record_steps")
        steps = min(int(self.rec["step"].item()), self.rec_capacity)
        out = {"steps": steps, "t0": self.rec_t0}
        for k, _ in self._REC_AGENT:
            out[k] = self.rec[k].view(self.n, self.rec_capacity)[:, :steps].cpu().numpy()
        for k, _ in self._REC_PATCH:
            out[k] = self.rec[k].view(max(self.np, 1), self.rec_capacity)[:self.np, :steps] \
                .cpu().numpy()
        out["soc_bits"] = self.rec["soc_bits"].view(self.n, self.rec_capacity, self.words)[
            :, :steps].cpu().numpy().view(np.uint32)
        out["radius"] = self.pt["radius"].cpu().numpy()
        return out

    def save_reference_json(self, folder: str, env: Optional[dict] = None):
        """Write agent_data.json, resource_data.json (and env_params.json when `env` is
        given) in the reference's RAM-recording layout (ifdb.save_ifdb_as_csv with
        as_zar=False, ifdb.py:412-434; env_saver.save_env_vars), readable by its DataLoader."""
        import json
        import os
        os.makedirs(folder, exist_ok=True)
        agents, resources = reference_json(self.recording(), self.params.rv)
        with open(os.path.join(folder, "agent_data.json"), "w") as f:
            f.write(agents)
        with open(os.path.join(folder, "resource_data.json"), "w") as f:
            f.write(resources)
        if env is not None:
            with open(os.path.join(folder, "env_params.json"), "w") as f:
                json.dump(dict(env), f, indent=4)

    def save_reference_zarr(self, folder: str, env: Optional[dict] = None,
                            save_extracted_vfield: bool = False):
        """Write the recording as the zarr arrays of the reference's save_ifdb_as_csv with
        as_zar=True (ifdb.py:435-536; USE_ZARR_FORMAT=1), plus env_params.json when `env` is
        given; save_extracted_vfield adds ag_vf, the social field rebuilt from its stored edges
        like the reference does."""
        import json
        import os
        rec = self.recording()
        agents = agents_dict(rec, self.params.rv) if save_extracted_vfield else \
            agents_dict({k: v for k, v in rec.items() if k != "soc_bits"}, self.params.rv)
        names = save_reference_zarr(folder, agents, resources_dict(rec), self.params.rv,
                                    save_extracted_vfield)
        if env is not None:
            with open(os.path.join(folder, "env_params.json"), "w") as f:
                json.dump(dict(env), f, indent=4)
        return names

    def _dev(self, a, dt):
        arr = np.ascontiguousarray(np.asarray(a, dt))
        if dt in (np.uint32, np.uint64):
            arr = arr.view(np.int32 if dt == np.uint32 else np.int64)
        return torch.as_tensor(arr, device=self.device).clone()

    def _launch(self, stream, uniforms=None) -> int:
        status = self.lib.abm_forage_step(
            ctypes.byref(self._agent_struct), self.n, ctypes.byref(self._patch_struct), self.np,
            ctypes.byref(self._cparams), _lib.u32ptr(self.soc_bits), _lib.i32ptr(self.scratch),
            _lib.dptr(uniforms), _lib.u64ptr(self.diag), ctypes.c_void_p(stream.cuda_stream))
        st = _lib.check(status, "abm_forage_step")
        if self.rec is not None:   # the reference records after the agents' update
            _lib.check(self.lib.abm_forage_record(
                ctypes.byref(self._agent_struct), self.n, ctypes.byref(self._patch_struct),
                self.np, _lib.u32ptr(self.soc_bits), int(self.params.rv),
                ctypes.byref(self._rec_struct), ctypes.c_void_p(stream.cuda_stream)),
                "abm_forage_record")
        return st

    def step(self, uniforms: Optional[torch.Tensor] = None, stream=None) -> int:
        """One step; `uniforms` (n float64 on the device) replaces the random-walk draws."""
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        st = self._launch(s, uniforms)
        self.t += 1
        return st

    def _warmup(self, stream):
        """One step on copies of the state: the library builds its lookup tables on first
        use, which must not happen inside a stream capture."""
        ag = {k: t.clone() for k, t in self.ag.items()}
        pt = {k: t.clone() for k, t in self.pt.items()}
        a_s = _lib.AbmForagerState(*[ctypes.cast(ag[k].data_ptr(), c)
                                     for k, c in _lib.FORAGER_FIELDS])
        p_s = _lib.AbmPatchState(*[ctypes.cast(pt[k].data_ptr(), c) for k, c in _lib.PATCH_FIELDS])
        soc, scr = torch.empty_like(self.soc_bits), torch.empty_like(self.scratch)
        stream.wait_stream(torch.cuda.current_stream(self.device))   # the copies are ready
        _lib.check(self.lib.abm_forage_step(
            ctypes.byref(a_s), self.n, ctypes.byref(p_s), self.np, ctypes.byref(self._cparams),
            _lib.u32ptr(soc), _lib.i32ptr(scr), None, None, ctypes.c_void_p(stream.cuda_stream)),
            "abm_forage_step")
        stream.synchronize()

    def capture(self, chunk: int = 100):
        """Capture `chunk` steps as a CUDA graph on a private stream."""
        self._stream = torch.cuda.Stream(self.device)
        self._warmup(self._stream)
        self._stream.wait_stream(torch.cuda.current_stream(self.device))
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=self._stream):
            for _ in range(chunk):
                self._launch(self._stream)
        self._graph, self._chunk = g, chunk
        torch.cuda.current_stream(self.device).wait_stream(self._stream)

    def run(self, steps: int, chunk: int = 100):
        """Advance `steps` steps: graph replays of `chunk` steps, then single steps."""
        if steps >= chunk and (self._graph is None or self._chunk != chunk):
            self.capture(chunk)
        while steps >= chunk:
            self._graph.replay()
            self.t += chunk
            steps -= chunk
        for _ in range(steps):
            self.step()

    def run_in_library(self, steps: int, graph_chunk: int = 100, stream=None) -> int:
        """Advance `steps` steps with one abm_forage_run call (the library captures and replays
        its own CUDA graph of graph_chunk steps on `stream`, a non-default one; recording, when
        enabled, after every step).  Same state as `steps` calls of step()."""
        s = stream if stream is not None else torch.cuda.Stream(self.device)
        if stream is None:
            s.wait_stream(torch.cuda.current_stream(self.device))
        st = _lib.check(self.lib.abm_forage_run(
            ctypes.byref(self._agent_struct), self.n, ctypes.byref(self._patch_struct), self.np,
            ctypes.byref(self._cparams), _lib.u32ptr(self.soc_bits), _lib.i32ptr(self.scratch),
            int(steps), int(graph_chunk),
            ctypes.byref(self._rec_struct) if self.rec is not None else None,
            _lib.u64ptr(self.diag), ctypes.c_void_p(s.cuda_stream)), "abm_forage_run")
        if stream is None:
            torch.cuda.current_stream(self.device).wait_stream(s)
        self.t += int(steps)
        return st

    def agents_numpy(self) -> dict:
        out = {}
        for k, dt in AGENT_FIELDS:
            a = self.ag[k].cpu().numpy()
            out[k] = a.view(dt) if dt in (np.uint32, np.uint64) else a
        return out

    def patches_numpy(self) -> dict:
        out = {}
        for k, dt in PATCH_FIELDS:
            a = self.pt[k].cpu().numpy()
            out[k] = a.view(dt) if dt in (np.uint32, np.uint64) else a
        return out

    def soc_numpy(self) -> np.ndarray:
        """(n, rv) uint8 social fields of the last step (stored order)."""
        words = self.soc_bits.cpu().numpy().view(np.uint32).astype("<u4").view(np.uint8)
        bits = np.unpackbits(words.reshape(self.n, -1), axis=1, bitorder="little")
        return bits[:, : self.params.rv]

    def collected(self) -> np.ndarray:
        return self.ag["collected"].cpu().numpy()


def efficiency(collected_start, collected_end, dt: float) -> np.ndarray:
    """Per-agent foraging efficiency (data_loader.py:1333-1346): units collected between two
    times divided by the elapsed time."""
    return (np.asarray(collected_end, np.float64) - np.asarray(collected_start, np.float64)) / dt
