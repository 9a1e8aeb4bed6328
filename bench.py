#!/usr/bin/env python3
"""Benchmark of the GB300 visual-flocking hot path (agent-steps/s).

Headline workload: the large single swarm -- N=4096 visual-flocking agents, radius 5,
5000x5000 walled arena, Rv=3600 over a 2*pi field of view, headings von Mises (kappa=2)
around a seeded mean, alpha0=beta0=1, alpha1=beta1=0.08, FP32 state, bitmask VPF.  One
bench step = one simulation timestep of the whole swarm (N agent-steps) through
abm_vpf_flock_step.  Inputs are seeded synthetic swarms (the reference publishes no dataset).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

`value` is kernel-only throughput with the state resident in HBM; `e2e` is the same metric
through the C-ABI call a per-step host loop makes (pinned host state -> H2D -> step ->
D2H every step).  The working set (~130 KB) is far below L2, so L2 is flushed (a 256 MiB
write) between timed steps and only the step itself is inside the CUDA events.
`--impl reference` times the reference algorithm's CPU restatement (the FP64 C port under
oracle/, all host threads) on a bounded sample of focal agents of the same workload.  The
`cpu_baseline` leg of the GPU arm times that port on one full step of the headline swarm (and
reports the GPU step's parity against it) and, when the reference is installed in
baseline/_ref, the reference's own numpy path (vf_supcalc.projection_field +
VSWRM_flocking_state_variables, unmodified, behind three import shims) on one core and on all
host cores.
Multi-GPU runs are independent replicas (the path does not shard across GPUs); the batched
sweep's instances are split across the ranks as disjoint sets.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "agent-steps/s"
WORKLOAD = dict(workload="vf_large_swarm", n_agents=4096, radius=5.0, arena=[5000.0, 5000.0],
                window_pad=30.0, rv=3600, fov="2pi", heading="von Mises kappa=2",
                alp0=1.0, bet0=1.0, alp1=0.08, bet1=0.08, gam=0.1, v0=1.0, boundary="walls",
                state="float32", vpf="bitmask", step="one timestep of all agents (Jacobi)",
                seed=2026)
# Frozen algorithmic work per agent-step (FP32 ops and MUFU ops), per ordered pair and per
# agent: F = 36 (N-1) + 4 Rv + 20, M = 3 (N-1).
F_PAIR, F_PX, F_UPD, M_PAIR = 36, 4, 20, 3
L2_FLUSH_BYTES = 256 << 20
# DRAM traffic of one launch of the dominant kernel (the group-form pair kernel) of this
# workload, from the ncu capture summarised in profiles/vpf_pairs_group_n4096_rv3600.md
# (dram__bytes_read.sum + dram__bytes_write.sum).
NCU_TRAFFIC_BYTES = 2009088


def make_workload(seed=WORKLOAD["seed"], n=WORKLOAD["n_agents"]):
    rng = np.random.default_rng(seed)
    W, H = WORKLOAD["arena"]
    R, pad = WORKLOAD["radius"], WORKLOAD["window_pad"]
    x = rng.uniform(pad - R, pad + W - R, n).astype(np.float32)
    y = rng.uniform(pad - R, pad + H - R, n).astype(np.float32)
    th = np.mod(rng.vonmises(rng.uniform(0, 2 * np.pi), 2.0, n), 2 * np.pi).astype(np.float32)
    v = np.zeros(n, np.float32)
    return {"x": x, "y": y, "theta": th, "v": v}


def make_params():
    from abm_gb300.params import VFParams
    W, H = WORKLOAD["arena"]
    return VFParams(gam=0.1, v0=1.0, alp0=1.0, alp1=0.08, bet0=1.0, bet1=0.08,
                    boundary="walls", width=W, height=H, window_pad=WORKLOAD["window_pad"],
                    fov=(-math.pi, math.pi), rv=WORKLOAD["rv"], radius=WORKLOAD["radius"])


def oracle_params_dict():
    W, H = WORKLOAD["arena"]
    return dict(gam=0.1, v0=1.0, alp0=1.0, alp1=0.08, alp2=0.0, bet0=1.0, bet1=0.08, bet2=0.0,
                boundary=0, limit_movement=0, max_vel=3.0, max_th=0.1, width=W, height=H,
                window_pad=WORKLOAD["window_pad"], fov0=-math.pi, fov1=math.pi,
                rv=WORKLOAD["rv"], radius=WORKLOAD["radius"], dt=1.0)


# ---------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": float(max(smax)) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------- peaks
def measure_peaks(lib, torch, stream):
    """Live FP32 (FFMA) and MUFU throughput of this GPU, in ops/s (best of 5)."""
    import ctypes
    from abm_gb300 import _lib
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    blocks = props.multi_processor_count * 8
    sink = torch.zeros(1024, dtype=torch.float32, device="cuda")
    out = {}
    for kind, name, iters in ((0, "fp32_ffma", 4096), (2, "fp32_ffma2", 2048),
                              (1, "mufu", 1024)):
        best = 0.0
        for _ in range(5):
            ops = ctypes.c_double()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _lib.check(lib.abm_probe_pipe_peak(kind, blocks, 256, iters, _lib.fptr(sink),
                                               ctypes.byref(ops),
                                               ctypes.c_void_p(stream.cuda_stream)))
            e1.record(stream)
            e1.synchronize()
            best = max(best, ops.value / (e0.elapsed_time(e1) * 1e-3))
        out[name] = best
    out["fp32"] = max(out["fp32_ffma"], out["fp32_ffma2"])   # the kernels issue both forms
    return out


# ---------------------------------------------------------------------- CPU baseline
def cpu_baseline(state, gpu=None):
    """The oracle's C port (the reference algorithm restated in FP64 C, OpenMP on all host
    threads) timed on one full snapshot step of the headline swarm -- every agent's VPF, VSWRM
    terms and update -- and the parity of the GPU's step of the same snapshot against it
    (`gpu`: the GPU step's vpf, terms, state and diagnostics); the same port on one core on a
    smaller sample; then the reference's own numpy path (reference_numpy_baseline)."""
    import oracle
    p = oracle_params_dict()
    threads = oracle.num_threads()
    n = len(state["x"])
    st64 = {k: np.asarray(state[k], np.float32).astype(np.float64) for k in state}
    t0 = time.perf_counter()
    ref = oracle.vf_step(st64, p, want_excuse=True)
    wall = time.perf_counter() - t0
    per_agent = wall / n
    n1 = int(max(1, min(n, 2.0 / max(per_agent * threads, 1e-6))))
    oracle.set_threads(1)
    try:
        t0 = time.perf_counter()
        oracle.vf_step_range(st64, p, 0, n1)
        wall1 = time.perf_counter() - t0
    finally:
        oracle.set_threads(threads)
    out = {"value": n / wall, "unit": METRIC, "cores": threads, "kind": "port",
           "sample": f"one full step of the N={n} snapshot ({wall:.1f} s wall): every agent's "
                     "VPF, VSWRM terms and update, FP64 C restatement with OpenMP",
           "host_cpus": os.cpu_count(), "cpu_model": cpu_model(),
           "one_core": {"value": n1 / wall1, "unit": METRIC,
                        "sample": f"{n1} focal agents x 1 step, one thread ({wall1:.1f} s)"}}
    if gpu is not None:
        bad = gpu["vpf"] != ref["vpf"]
        unexcused = bad & (ref["excuse"] == 0)
        scale = np.maximum(np.abs(ref["terms"]), 1e-6)
        ulps = {}
        for k in ("x", "y", "theta", "v"):
            r32 = ref[k].astype(np.float32)
            ulp = np.spacing(np.abs(r32)).astype(np.float64)
            ulps[k] = float(np.max(np.abs(gpu["state"][k].astype(np.float64) - ref[k]) / ulp))
        out["parity_of_gpu_step"] = {
            "agents": n,
            "vpf_mismatched_pixels": int(bad.sum()),
            "vpf_mismatched_agents": int(bad.any(axis=1).sum()),
            "vpf_pixels_outside_excuse_mask": int(unexcused.sum()),
            "excused_pixels_possible": int(ref["excuse"].sum()),
            "near_boundary_pairs_oracle": int(ref["near"].sum()),
            "near_boundary_pairs_kernel": int(gpu["diag"]["near_boundary"]),
            "pairs_redecided_kernel": int(gpu["diag"]["pairs_resolved"]),
            "terms_max_rel_err": float(np.max(np.abs(gpu["terms"] - ref["terms"]) / scale)),
            "state_max_ulps": ulps,
            "bar": "VPF exact outside the oracle's excuse mask (pixels that pairs within 1e-9 rad "
                   "of a decision boundary flip); terms 1e-5 relative; state 2 float32 ulps"}
    out["reference_numpy"] = reference_numpy_baseline(state)
    return out


def cpu_model():
    try:
        r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10)
        for ln in r.stdout.splitlines():
            if ln.strip().startswith("Model name"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return None


# ---------------------------------------------------------------------- reference numpy path
REF_ROOT = os.path.join(ROOT, "baseline", "_ref")


def _reference_vf_supcalc():
    """vf_supcalc of the reference installed in baseline/_ref, imported unmodified behind the
    three shims its import needs here: a stub `dotenv` (python-dotenv is absent; the module
    reads no .env keys on this path), and scipy.integrate.trapz restated as np.trapezoid (the
    same trapezoid rule; trapz was removed from SciPy)."""
    import types
    sys.dont_write_bytecode = True
    if REF_ROOT not in sys.path:
        sys.path.insert(0, REF_ROOT)
    if "dotenv" not in sys.modules:
        stub = types.ModuleType("dotenv")
        stub.dotenv_values = lambda *a, **k: {}
        sys.modules["dotenv"] = stub
    import scipy.integrate
    if not hasattr(scipy.integrate, "trapz"):
        scipy.integrate.trapz = (lambda y, x=None, dx=1.0, axis=-1:
                                 np.trapezoid(y, x=x, dx=dx, axis=axis))
    from abm.projects.visual_flocking.vf_agent import vf_supcalc
    return vf_supcalc


class _RefVfParams:
    """The duck-typed vf_params module object VSWRM_flocking_state_variables reads."""
    GAM, V0 = WORKLOAD["gam"], WORKLOAD["v0"]
    ALP0, ALP1, ALP2 = WORKLOAD["alp0"], WORKLOAD["alp1"], 0.0
    BET0, BET1, BET2 = WORKLOAD["bet0"], WORKLOAD["bet1"], 0.0


_REF_STATE = None


def _ref_worker_init(state):
    global _REF_STATE
    _REF_STATE = state
    _reference_vf_supcalc()


def _ref_agent_step(vfs, st, i, phi):
    """One agent-step of the reference path, as VFAgent.calc_soc_v_proj (vf_agent.py:216-237)
    and perform_action / update_agent_position (:263-309) call it: projection_field over every
    other agent, the binarised sum, VSWRM on the flipped field, the heading / speed / position
    update."""
    n = len(st["x"])
    W, H = WORKLOAD["arena"]
    R = WORKLOAD["radius"]
    others = [j for j in range(n) if j != i]
    vfield = vfs.projection_field(
        fov=(-math.pi, math.pi), v_field_resolution=WORKLOAD["rv"],
        position=np.array([st["x"][i], st["y"][i]]), radius=R, orientation=st["theta"][i],
        object_positions=[np.array([st["x"][j], st["y"][j]]) for j in others],
        object_sizes=[R for _ in others], boundary_cond="walls", arena_width=W,
        arena_height=H, ag_id=i)
    sv = vfield.sum(axis=0)
    sv[sv > 0] = 1
    dv, dphi = vfs.VSWRM_flocking_state_variables(st["v"][i], phi, np.flip(sv), _RefVfParams)
    th = st["theta"][i] + dphi
    th = th + 2 * np.pi if th < 0 else (th - 2 * np.pi if th > 2 * np.pi else th)
    v = st["v"][i] + dv
    return st["x"][i] + v * np.cos(th), st["y"][i] - v * np.sin(th), th, v


def _ref_task(args):
    idx, reps = args
    vfs = _reference_vf_supcalc()
    phi = np.arange(-np.pi, np.pi, (2 * np.pi) / WORKLOAD["rv"])
    t0 = time.perf_counter()
    for _ in range(reps):
        for i in idx:
            _ref_agent_step(vfs, _REF_STATE, int(i), phi)
    return time.perf_counter() - t0


def reference_numpy_baseline(state, focal=64, reps=3, one_core_agents=12):
    """The reference's own numpy path (baseline/_ref) on the headline snapshot: `focal` seeded
    focal agents x `reps` steps from the snapshot over a multiprocessing pool of all host
    cores (spawn), and `one_core_agents` agent-steps in this process on one core; per
    agent-step cost at the full N, so agent-steps/s needs no extrapolation in N."""
    if not os.path.isdir(os.path.join(REF_ROOT, "abm")):
        return {"unavailable": "the reference is not installed in baseline/_ref (pip install "
                               "--no-deps --target baseline/_ref <reference source tree>)"}
    import concurrent.futures as cf
    import multiprocessing as mp
    st = {k: np.asarray(state[k], np.float64) for k in ("x", "y", "theta", "v")}
    n = len(st["x"])
    rng = np.random.default_rng(WORKLOAD["seed"] + 1)
    idx = np.sort(rng.choice(n, focal, replace=False))
    cores = os.cpu_count() or 1
    try:
        global _REF_STATE
        _REF_STATE = st
        vfs = _reference_vf_supcalc()
        phi = np.arange(-np.pi, np.pi, (2 * np.pi) / WORKLOAD["rv"])
        _ref_agent_step(vfs, st, int(idx[0]), phi)          # warm-up (imports, caches)
        t0 = time.perf_counter()
        for i in idx[:one_core_agents]:
            _ref_agent_step(vfs, st, int(i), phi)
        t1 = time.perf_counter() - t0
        chunks = [(list(idx[k::cores]), reps) for k in range(min(cores, focal))]
        # spawned workers (a pool forked from a process that uses CUDA can hang); a worker
        # that dies breaks the pool with an error instead of being replaced
        with cf.ProcessPoolExecutor(max_workers=len(chunks), mp_context=mp.get_context("spawn"),
                                    initializer=_ref_worker_init, initargs=(st,)) as pool:
            list(pool.map(_ref_task, [([int(idx[0])], 1)] * len(chunks)))   # warm the workers
            t0 = time.perf_counter()
            list(pool.map(_ref_task, chunks))
            tp = time.perf_counter() - t0
    except Exception as e:   # the baseline is reported, never required
        return {"unavailable": f"reference numpy path failed: {type(e).__name__}: {e}"}
    return {"kind": "reference", "unit": METRIC, "host_cpus": cores, "cpu_model": cpu_model(),
            "path": "abm/projects/visual_flocking/vf_agent/vf_supcalc.py projection_field + "
                    "VSWRM_flocking_state_variables per agent as VFAgent calls them "
                    "(vf_agent.py:216-309), shimmed (stub dotenv, scipy.integrate.trapz = "
                    "np.trapezoid), unmodified",
            "all_cores": {"value": focal * reps / tp, "cores": len(chunks),
                          "sample": f"{focal} seeded focal agents x {reps} steps from the N={n} "
                                    f"snapshot over a spawn Pool of {len(chunks)} processes "
                                    f"({tp:.1f} s wall)"},
            "one_core": {"value": one_core_agents / t1, "cores": 1,
                         "sample": f"{one_core_agents} focal agents x 1 step, one process "
                                   f"({t1:.1f} s)"}}


def run_reference(args, rank, world):
    if rank != 0:
        return
    import oracle
    state = make_workload()
    p = oracle_params_dict()
    threads = oracle.num_threads()
    t0 = time.perf_counter()
    oracle.vf_step_range(state, p, 0, threads)
    per_round = time.perf_counter() - t0        # one agent per thread
    budget = 150.0 / max(args.steps + args.warmup, 1)
    per_step = max(threads, int(budget / max(per_round, 1e-6)) * threads)
    per_step = min(per_step, len(state["x"]))
    for _ in range(args.warmup):
        oracle.vf_step_range(state, p, 0, per_step)
    t0 = time.perf_counter()
    for s in range(args.steps):
        i0 = (s * per_step) % max(len(state["x"]) - per_step + 1, 1)
        oracle.vf_step_range(state, p, i0, i0 + per_step)
    wall = time.perf_counter() - t0
    value = per_step * args.steps / wall
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": wall * 1e3 / max(args.steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(WORKLOAD), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": METRIC, "cores": threads, "kind": "port",
                             "sample": f"{per_step} focal agents per step of the N=4096 "
                                       "snapshot; FP64 C restatement of the reference path "
                                       "(oracle/vpf_oracle.c), OpenMP"},
            "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------- batched sweep leg
BATCHED = dict(workload="vf_batched_sweep", n_instances=512, n_per_instance="uniform int [10,500]",
               alp0_bet0="16 x 32 grid over [0.1, 3]", rv=1200, radius=10.0,
               arena=[1000.0, 1000.0], boundary="walls", steps=2000, graph_chunk=100, seed=3,
               torus_steps=1000)


def compact_table(tried):
    """[mode, warps per agent, chunks, agents per block, tile, us per step] per candidate."""
    return {"columns": ["mode", "warps_per_agent", "chunks", "warps_per_block", "tile",
                        "us_per_step"],
            "rows": [[t["mode"], t["warps_per_agent"], t["chunks"], t["warps_per_block"],
                      t["tile"], round(t["ms_per_step"] * 1e3, 2)] for t in tried]}


# the library's default step configuration: automatic form and neighbour chunks
DEFAULT_STEP_CONFIG = {"mode": 0, "warps_per_agent": 1, "warps_per_block": 8, "tile": 8192,
                       "chunks": 0}


def batched_leg(torch, lib, stream, steps=BATCHED["steps"], flush=None, rank=0, world=1,
                device=None):
    """Batched sweep: 512 instances advanced by one abm_vpf_flock_batched call per step,
    captured in CUDA graphs of 100 steps; compared with per-instance abm_vpf_flock_step calls
    (eager, and captured as a graph of 512 x 2 launches per step).  With several ranks each
    runs a disjoint share of the instances (balanced by pair work) and the times combine as
    the slowest rank's, the agent-steps as their sum."""
    import ctypes
    from abm_gb300 import _lib
    from abm_gb300 import autotune
    from abm_gb300.batched import BatchedSweep, sweep_instances
    from abm_gb300.params import VFParams
    from abm_gb300.replicas import combine, shard_instances
    vp = VFParams(gam=0.1, v0=1.0, alp1=0.08, bet1=0.08, width=1000.0, height=1000.0,
                  rv=BATCHED["rv"], radius=BATCHED["radius"])
    inst = sweep_instances(n_instances=BATCHED["n_instances"], seed=BATCHED["seed"])
    all_sizes = np.array([len(d["x"]) for d in inst])
    mine = shard_instances(all_sizes, world, rank)
    inst = [inst[k] for k in mine]
    b = BatchedSweep(vp, inst)
    tuned = autotune.tune(b, reps=3)     # warps per agent of the segmented L1 form
    chunk = BATCHED["graph_chunk"]
    b.capture(chunk)
    b.run(chunk, chunk=chunk)                       # warm-up replay
    torch.cuda.synchronize()
    ev = []
    done = 0
    while done < steps:
        if flush is not None:
            flush.fill_(float(done))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        b.run(chunk, chunk=chunk)
        e1.record()
        ev.append((e0, e1))
        done += chunk
    torch.cuda.synchronize()
    t_b = sum(a.elapsed_time(c) for a, c in ev) * 1e-3
    agent_steps = b.n * done

    # per-instance launches of the plain step (views into one concatenated state)
    n_tot, offs = b.n, b.offsets
    bufs = [{k: t.clone() for k, t in b._bufs[b._cur].items()},
            {k: torch.empty_like(t) for k, t in b._bufs[b._cur].items()}]
    cp = vp.to_c()
    ov_t = b.ov_tensors

    def per_instance_step(src, s):
        for k in range(len(offs) - 1):
            a0, a1 = int(offs[k]), int(offs[k + 1])
            sl = lambda d: _lib.AbmSwarmState(*[_lib.fptr(d[key][a0:a1])
                                                for key in ("x", "y", "theta", "v")])
            ov = _lib.AbmAgentOverrides(None, _lib.fptr(ov_t["alp0"][a0:a1]),
                                        _lib.fptr(ov_t["bet0"][a0:a1]), None)
            si, so = sl(bufs[src]), sl(bufs[1 - src])
            _lib.check(lib.abm_vpf_flock_step(ctypes.byref(si), ctypes.byref(so), a1 - a0,
                                              ctypes.byref(cp), ctypes.byref(ov), None, None,
                                              None, ctypes.c_void_p(s.cuda_stream)))

    autotune.apply(DEFAULT_STEP_CONFIG)     # per-instance launches: the automatic choice
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        per_instance_step(0, s)                     # warm-up (workspace, tables)
        s.synchronize()
        k_eager = 10
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for k in range(k_eager):
            per_instance_step(k % 2, s)
        e1.record(s)
        e1.synchronize()
        t_eager = e0.elapsed_time(e1) * 1e-3 / k_eager
        g = torch.cuda.CUDAGraph()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.graph(g, stream=s):
            per_instance_step(0, s)
            per_instance_step(1, s)
        reps = 20
        g.replay()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            g.replay()
        e1.record(s)
        e1.synchronize()
        t_graph = e0.elapsed_time(e1) * 1e-3 / (2 * reps)
    torch.cuda.current_stream().wait_stream(s)

    # the same instances on a 1000 x 1000 torus (the boundary of the reference's current sweep
    # experiments), automatic configuration, timed the same way
    vt = VFParams(gam=0.1, v0=1.0, alp1=0.08, bet1=0.08, width=1000.0, height=1000.0,
                  rv=BATCHED["rv"], radius=BATCHED["radius"], boundary="infinite")
    bt = BatchedSweep(vt, inst)
    bt.capture(chunk)
    bt.run(chunk, chunk=chunk)                      # warm-up replay
    torch.cuda.synchronize()
    ev = []
    done_t = 0
    while done_t < BATCHED["torus_steps"]:
        if flush is not None:
            flush.fill_(float(done_t))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        bt.run(chunk, chunk=chunk)
        e1.record()
        ev.append((e0, e1))
        done_t += chunk
    torch.cuda.synchronize()
    t_t = sum(a.elapsed_time(c) for a, c in ev) * 1e-3
    (t_t,), torus_agent_steps = combine([t_t], bt.n * done_t, device=device)

    (t_b, t_eager, t_graph), agent_steps = combine([t_b, t_eager, t_graph], agent_steps,
                                                   device=device)
    n_tot = agent_steps // done
    per_step = t_b / done
    return {"workload": dict(BATCHED, total_agents=n_tot,
                             pairs_per_step=int((all_sizes.astype(np.int64) ** 2).sum()),
                             l2="flushed between 100-step graph replays",
                             sharding=(f"{world} ranks, disjoint instance sets balanced by "
                                       "N_i^2" if world > 1 else "single rank")),
            "value": agent_steps / t_b, "unit": METRIC, "ms_per_step": per_step * 1e3,
            "steps": done, "gpu_launches": 2 * done,
            "per_instance_launches": {"eager_value": n_tot / t_eager,
                                      "graph_value": n_tot / t_graph,
                                      "ms_per_step_eager": t_eager * 1e3,
                                      "ms_per_step_graph": t_graph * 1e3,
                                      "launches_per_step": 2 * BATCHED["n_instances"],
                                      "per_rank": "each rank launches its own instances"
                                                  if world > 1 else None},
            "speedup_vs_per_instance_graph": t_graph / per_step,
            "torus": {"boundary": "infinite", "config": "automatic", "steps": done_t,
                      "value": torus_agent_steps / t_t, "unit": METRIC,
                      "ms_per_step": t_t / done_t * 1e3, "gpu_launches": 2 * done_t},
            "autotune": {"best": tuned["best"], "table": compact_table(tuned["tried"])}}


# ---------------------------------------------------------------------- foraging leg
FORAGE = dict(workload="collective_foraging", n_agents=100, radius=10.0, arena=[1000.0, 1000.0],
              n_patches=3, patch_radius=30.0, patch_units=1000, quality=1.0, consumption=1.0,
              rv=1200, agent_fov=0.5, vision_range=2000.0, visual_exclusion=True,
              teleport=False, pooling_time=0, steps=10000, graph_chunk=100, seed=5,
              step="resource interaction + social VPF + decision/motion update (3 launches)")


# the same arena with agent-agent collisions on (AGENT_AGENT_COLLISION=1, ghost mode on)
FORAGE_COLLIDE = dict(FORAGE, workload="collective_foraging_collisions", steps=2000,
                      collide_agents=True, ghost_mode=True,
                      step="agent-agent collisions + resource interaction + social VPF + "
                           "decision/motion update (4 launches)")


def forage_params(collide=False):
    from abm_gb300.foraging import ForageParams
    return ForageParams(width=1000.0, height=1000.0, agent_radius=10.0, patch_radius=30.0,
                        min_resc_units=1000, max_resc_units=1001, min_resc_quality=1.0,
                        max_resc_quality=1.0, consumption=1.0, rv=1200, fov=0.5,
                        vision_range=2000.0, visual_exclusion=True, teleport_exploit=False,
                        pooling_time=0, seed=FORAGE["seed"], collide_agents=collide,
                        ghost_mode=True)


def forage_leg(torch, steps=FORAGE["steps"], with_cpu=True, collide=False):
    """The foraging workload run for `steps` steps in CUDA graphs of 100 steps; foraging
    efficiency (units per agent per step, data_loader.py:1333-1346) over the run; the oracle
    step on the host for a bounded sample of steps.  collide: agent-agent collisions on."""
    from abm_gb300.foraging import ForagingSim, efficiency
    prm = forage_params(collide)
    sim = ForagingSim(prm, n_agents=FORAGE["n_agents"], n_patches=FORAGE["n_patches"],
                      init_seed=FORAGE["seed"])
    chunk = FORAGE["graph_chunk"]
    sim.run(chunk, chunk=chunk)                     # capture + one warm-up replay
    torch.cuda.synchronize()
    c0, t0 = sim.collected(), sim.t
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    sim.run(steps, chunk=chunk)
    e1.record()
    e1.synchronize()
    t = e0.elapsed_time(e1) * 1e-3
    eff = efficiency(c0, sim.collected(), sim.t - t0)
    n = FORAGE["n_agents"]
    out = {"workload": FORAGE_COLLIDE if collide else FORAGE, "value": n * steps / t,
           "unit": METRIC, "ms_per_step": t / steps * 1e3, "steps": steps,
           "gpu_launches": (4 if collide else 3) * steps,
           "efficiency_mean": float(eff.mean()), "efficiency_max": float(eff.max()),
           "diagnostics": {"nonfinite": int(sim.diag[2].item()),
                           "failed_regenerations": int(sim.diag[4].item())}}
    if collide:
        out["agents_in_collide_mode_at_end"] = int(np.sum(sim.agents_numpy()["override_mode"]
                                                          == 4))
    if with_cpu:
        import oracle
        fp, ip, seed = prm.oracle_arrays()
        ag, pt = sim.agents_numpy(), sim.patches_numpy()
        k, t_cpu = 0, 0.0
        while t_cpu < (5.0 if collide else 10.0) and k < 400:
            a = time.perf_counter()
            ag, pt, _, _ = oracle.forage_step(ag, pt, fp, ip, seed)
            t_cpu += time.perf_counter() - a
            k += 1
        out["cpu_baseline"] = {"value": n * k / t_cpu, "unit": METRIC, "cores": 1,
                               "kind": "port", "sample": f"{k} steps of the same arena, FP64 C "
                                                         "restatement, one thread"}
    return out


# ---------------------------------------------------------------------- metarunner leg
METARUNNER = dict(workload="metarunner_grid", criteria=["Tunable VF_ALP0 linspace(0.1, 3, 16)",
                                                         "Tunable VF_BET0 linspace(0.1, 3, 32)",
                                                         "Constant N 100"],
                  num_batches=1, arena=[1000.0, 1000.0], rv=1200, radius=10.0, steps=1000,
                  graph_chunk=100, seed=1)


def metarunner_leg(torch):
    """A metarunner sweep (the reference's MetaProtocol definitions) run end to end through
    abm_gb300.metarunner.BatchedProtocol.run: expansion, initial states, batched launches in
    graphs of 100 steps and the final states back on the host, timed by the wall clock."""
    from abm_gb300 import metarunner as mr
    base = {"ENV_WIDTH": "1000", "ENV_HEIGHT": "1000", "VISUAL_FIELD_RESOLUTION": "1200",
            "RADIUS_AGENT": "10", "VF_ALP1": "0.08", "VF_BET1": "0.08"}
    bp = mr.BatchedProtocol(base, num_batches=METARUNNER["num_batches"])
    bp.add_criterion(mr.Tunable("VF_ALP0", 0.1, 3.0, 16))
    bp.add_criterion(mr.Tunable("VF_BET0", 0.1, 3.0, 32))
    bp.add_criterion(mr.Constant("N", 100))
    steps = METARUNNER["steps"]
    bp.run(steps // 10, seed=METARUNNER["seed"])   # warm-up (tables, workspace)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = bp.run(steps, seed=METARUNNER["seed"], chunk=METARUNNER["graph_chunk"])
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    agents = sum(len(r["x"]) for r in res)
    return {"workload": METARUNNER, "configurations": len(res), "groups": len(bp.groups()),
            "value": agents * steps / t, "unit": METRIC, "wall_s": t,
            "timing": "wall clock of BatchedProtocol.run (setup, capture, launches, results)"}


# ---------------------------------------------------------------------- differentiable leg
ADJOINT = dict(workload="vf_differentiable", n_agents=256, radius=10.0, arena=[1500.0, 1500.0],
               steps=200, dt=0.1, checkpoint=20,
               loss="1 - polarisation + MSE(mean position, seeded target)",
               wrt="alp0, alp1, bet0, bet1, v0 and initial x, y, theta", seed=11)


def adjoint_leg(torch):
    """Edge-form rollout of the differentiable workload: forward only vs forward + adjoint
    (gradients of the loss w.r.t. the five parameters and the initial state), best of 3 wall
    times with the device synchronised, in the float32 and the FP64 kernels."""
    import time as _t
    from abm_gb300 import edge
    from abm_gb300.params import VFParams
    W = ADJOINT["arena"][0]
    n, steps = ADJOINT["n_agents"], ADJOINT["steps"]
    rng = np.random.default_rng(ADJOINT["seed"])
    x0 = rng.uniform(30, 30 + W - 20, n)
    y0 = rng.uniform(30, 30 + W - 20, n)
    th0 = rng.uniform(0, 2 * np.pi, n)
    base = VFParams(gam=0.1, v0=1.0, alp0=1.0, alp1=0.08, bet0=1.0, bet1=0.08, width=W,
                    height=W, window_pad=30.0, radius=ADJOINT["radius"], dt=ADJOINT["dt"],
                    rv=1200)
    target = (0.45 * W, 0.55 * W)
    out = {}
    for name, dtype in (("fp32", torch.float32), ("fp64", torch.float64)):
        def make(grad):
            p = torch.tensor([1.0, 0.08, 1.0, 0.08, 1.0], dtype=torch.float64, device="cuda",
                             requires_grad=grad)
            init = [torch.tensor(a, dtype=dtype, device="cuda", requires_grad=grad)
                    for a in (x0, y0, th0, np.zeros(n))]
            return p, init

        def fwd():
            p, init = make(False)
            with torch.no_grad():
                edge.rollout(p, *init, base=base, steps=steps,
                             checkpoint=ADJOINT["checkpoint"])

        def fwd_bwd():
            p, init = make(True)
            o = edge.rollout(p, *init, base=base, steps=steps, checkpoint=ADJOINT["checkpoint"])
            L = edge.flocking_loss(o[0], o[1], o[2],
                                   torch.tensor(target, dtype=dtype, device="cuda"))
            L.backward()

        times = {}
        for label, fn in (("fwd", fwd), ("fwd_adjoint", fwd_bwd)):
            fn()
            torch.cuda.synchronize()
            best = float("inf")
            for _ in range(3):
                t0 = _t.perf_counter()
                fn()
                torch.cuda.synchronize()
                best = min(best, _t.perf_counter() - t0)
            times[label] = best
        out[name] = {"fwd_agent_steps_per_s": n * steps / times["fwd"],
                     "fwd_adjoint_agent_steps_per_s": n * steps / times["fwd_adjoint"],
                     "fwd_ms": times["fwd"] * 1e3, "fwd_adjoint_ms": times["fwd_adjoint"] * 1e3,
                     "cost_ratio_fwd_adjoint_over_fwd": times["fwd_adjoint"] / times["fwd"],
                     "gpu_launches": {"fwd": steps,
                                      "fwd_adjoint": 2 * steps + steps}}
    return {"workload": ADJOINT, "unit": METRIC, **out,
            "timing": "wall clock, device synchronised, best of 3 (includes host launch loop)"}


# ---------------------------------------------------------------------- GPU arm
def run_gb300(args, rank, world):
    import torch
    import torch.distributed as dist
    from abm_gb300 import _lib
    from abm_gb300.swarm import VFSwarm, step_host

    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = _lib.load()
    stream = torch.cuda.current_stream(dev)
    params = make_params()
    state = make_workload()
    n = len(state["x"])
    sw = VFSwarm(params, state["x"], state["y"], state["theta"], state["v"], device=dev)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    from abm_gb300 import autotune
    tuned = autotune.tune(sw, reps=5)   # launch configuration of the step, before any timing
    # The tuner times back-to-back steps with the state warm in L2; the timed region below
    # flushes L2 before every step.  Its best three candidates and the library's automatic
    # choice are timed again under those conditions, and the fastest is used.
    ran = sorted([t for t in tuned["tried"] if t["ms_per_step"] > 0],
                 key=lambda t: t["ms_per_step"])[:3]
    finalists = [dict(DEFAULT_STEP_CONFIG, chosen="automatic")] + [dict(t) for t in ran]
    for cfg in finalists:
        autotune.apply(cfg)
        for _ in range(3):
            sw.step()
        evs = []
        for k in range(20):
            flush.fill_(float(k))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sw.step()
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        cfg["ms_per_step_l2_flushed"] = float(np.mean([a.elapsed_time(c) for a, c in evs]))
    chosen = min(finalists, key=lambda c: c["ms_per_step_l2_flushed"])
    autotune.apply(chosen)
    sw.set_state(state["x"], state["y"], state["theta"], state["v"])

    peaks = measure_peaks(lib, torch, stream)
    for _ in range(args.warmup):
        sw.step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    clocks = ClockSampler(local)
    clocks.start()
    # ---- kernel-only timed region (state resident in HBM): K steps, each between CUDA events
    #      with the L2 flushed before it, bracketed by a barrier and a device synchronisation;
    #      the whole K-step sequence is repeated until about a second of step time has
    #      accumulated (the same repeat count on every rank), and the median repeat is reported
    def timed_sequence(step):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        barrier()
        for k in range(args.steps):
            flush.fill_(float(k))
            ev[k][0].record(stream)
            step(k)
            ev[k][1].record(stream)
        barrier()
        return float(sum(a.elapsed_time(b) for a, b in ev)) * 1e-3

    def repeats_for(first_s):
        r = max(1, min(args.max_repeats, int(math.ceil(args.min_device_s / max(first_s, 1e-9)))))
        if world > 1:
            import torch.distributed as dist
            t = torch.tensor([r], dtype=torch.int64, device=dev)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            r = int(t.item())
        return r

    step_kernel = lambda k: sw.step()
    t_wall0 = time.perf_counter()
    first = timed_sequence(step_kernel)
    reps_k = [first] + [timed_sequence(step_kernel) for _ in range(repeats_for(first) - 1)]
    t_wall = time.perf_counter() - t_wall0
    kernel_s = float(np.median(reps_k))

    # ---- end-to-end through the C-ABI with host buffers (host state in, host state out
    #      every step: abm_vpf_flock_step_host), timed the same way
    host_in = {k: torch.from_numpy(state[k].copy()).pin_memory() for k in state}
    host_out = {k: torch.empty(n, dtype=torch.float32).pin_memory() for k in state}
    cparams = params.to_c()
    for _ in range(args.warmup):
        step_host(lib, cparams, n, host_in, host_out, stream)
    bufs = [host_in, host_out]

    def step_e2e(k):
        step_host(lib, cparams, n, bufs[0], bufs[1], stream)
        bufs.reverse()

    first = timed_sequence(step_e2e)
    reps_e = [first] + [timed_sequence(step_e2e) for _ in range(repeats_for(first) - 1)]
    e2e_s = float(np.median(reps_e))
    clk = clocks.stop()

    # the GPU's step of the pristine snapshot, for the parity summary of the CPU leg
    ref_sw = VFSwarm(params, state["x"], state["y"], state["theta"], state["v"], device=dev)
    ref_sw.step(want_vpf=True, want_terms=True)
    ref_sw.check_status()
    gpu_step = {"vpf": ref_sw.vpf_numpy(), "terms": ref_sw.terms.cpu().numpy(),
                "state": ref_sw.state_numpy(), "diag": ref_sw.diagnostics()}
    sw.check_status()
    # batched sweep on every rank (each its share of the instances), before rank 0 reports
    batched = (None if args.no_batched else
               batched_leg(torch, lib, stream, flush=flush, rank=rank, world=world, device=dev))

    from abm_gb300.replicas import combine
    (kernel_s, e2e_s), agent_steps = combine([kernel_s, e2e_s], n * args.steps, device=dev)
    if rank != 0:
        return

    value = agent_steps / kernel_s
    e2e_value = agent_steps / e2e_s
    t_launch = kernel_s / args.steps
    rv = WORKLOAD["rv"]
    F = n * (F_PAIR * (n - 1) + F_PX * rv + F_UPD)
    M = n * M_PAIR * (n - 1)
    frac_f = F / t_launch / peaks["fp32"]
    frac_m = M / t_launch / peaks["mufu"]
    bound = "fp32" if frac_f >= frac_m else "mufu"
    achieved = (F if bound == "fp32" else M) / t_launch
    peak = peaks[bound]
    roofline = {"bound": bound, "achieved": achieved / 1e12, "peak": peak / 1e12,
                "unit": "TFLOP/s" if bound == "fp32" else "Tops/s (MUFU)",
                "frac": achieved / peak,
                "traffic": NCU_TRAFFIC_BYTES,
                "timed": "whole step on the launching stream: the pair kernel and its "
                         "dependent finish kernel (the group-form pair kernel is ~83 % of the "
                         "serialised launch list)",
                "algorithmic": {"fp32_ops_per_launch": F, "mufu_ops_per_launch": M,
                                "fp32_frac": frac_f, "mufu_frac": frac_m,
                                "hbm_bytes_per_launch": n * 32},
                "peak_source": "measured live in this run: FFMA, packed FFMA2 and MUFU.RSQ "
                               "chain probes (abm_probe_pipe_peak), best of 5; fp32 peak = "
                               "the higher of FFMA and FFMA2",
                "peaks_measured": {k: v / 1e12 for k, v in peaks.items()},
                "kernel_ms_mean": t_launch * 1e3,
                "kernel_ms_repeats_min_max": [min(reps_k) / args.steps * 1e3,
                                              max(reps_k) / args.steps * 1e3]}
    diag = sw.diagnostics()
    line = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_launch * 1e3,
            "repeats": len(reps_k),
            "timing": f"{args.steps} steps per timed sequence (CUDA events per step, L2 flushed "
                      f"before each), the sequence repeated {len(reps_k)} times (about "
                      f"{args.min_device_s:g} s of step time); value and ms_per_step from the "
                      "median sequence, max over ranks",
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded swarm; the reference publishes no dataset)",
            "config": dict(WORKLOAD, parallelism="replicas" if world > 1 else "single",
                           l2="flushed between timed steps (256 MiB write)"),
            "e2e": {"value": e2e_value, "unit": METRIC, "h2d_bytes_per_step": 16 * n,
                    "d2h_bytes_per_step": 16 * n, "repeats": len(reps_e),
                    "path": "abm_vpf_flock_step_host via ctypes on pinned host state: the "
                            "input gathered from host memory by one kernel, the new state "
                            "written to host memory by the step's last kernel, every step"},
            # pair kernel + finish (or update) kernel per step, in every timed sequence
            "gpu_launches": 2 * args.steps * len(reps_k),
            "roofline": roofline, "clocks": clk,
            "launch_config": dict(chosen, chosen_by="abm_vpf_autotune (5 back-to-back steps "
                                  "per candidate), then its best three and the automatic "
                                  "choice timed over 20 steps with the L2 flushed before each",
                                  candidates=len(tuned["tried"]),
                                  finalists=[{k: f[k] for k in ("mode", "warps_per_agent",
                                                                "chunks",
                                                                "ms_per_step_l2_flushed")}
                                             for f in finalists],
                                  table=compact_table(tuned["tried"])),
            "wall_s_timed_region": t_wall,
            "diagnostics": diag}
    if batched is not None:
        line["batched"] = batched
    if not args.no_adjoint:
        line["adjoint"] = adjoint_leg(torch)
    if not args.no_forage:
        line["forage"] = forage_leg(torch, with_cpu=not args.no_cpu_baseline)
        line["forage_collisions"] = forage_leg(torch, steps=FORAGE_COLLIDE["steps"],
                                               with_cpu=not args.no_cpu_baseline, collide=True)
    if not args.no_batched:
        line["metarunner"] = metarunner_leg(torch)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(state, gpu_step)
    print(json.dumps(line), flush=True)


def profile_workload(which: str):
    """A few eager steps of one leg's workload and nothing else: the command the ncu
    summaries under profiles/ capture (launch lists and single-kernel captures)."""
    import torch
    if which == "headline":
        from abm_gb300.swarm import VFSwarm
        st = make_workload()
        sw = VFSwarm(make_params(), st["x"], st["y"], st["theta"], st["v"])
        flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
        for k in range(10):   # as in the timed region: the L2 flushed before every step
            flush.fill_(float(k))
            sw.step()
    elif which in ("batched", "batched_torus"):
        from abm_gb300.batched import BatchedSweep, sweep_instances
        from abm_gb300.params import VFParams
        B = BATCHED
        vp = VFParams(gam=0.1, v0=1.0, alp1=0.08, bet1=0.08, width=1000.0, height=1000.0,
                      rv=B["rv"], radius=B["radius"],
                      boundary="infinite" if which == "batched_torus" else "walls")
        b = BatchedSweep(vp, sweep_instances(n_instances=B["n_instances"], seed=B["seed"]))
        for _ in range(8):
            b.step()
    elif which in ("forage", "forage_collide"):
        from abm_gb300.foraging import ForagingSim
        sim = ForagingSim(forage_params(which == "forage_collide"), n_agents=FORAGE["n_agents"],
                          n_patches=FORAGE["n_patches"], init_seed=FORAGE["seed"])
        for _ in range(300):
            sim.step()
    elif which == "edge":
        from abm_gb300 import edge
        from abm_gb300.params import VFParams
        A = ADJOINT
        rng = np.random.default_rng(A["seed"])
        n, (W, H) = A["n_agents"], A["arena"]
        t = lambda a: torch.tensor(a, dtype=torch.float32, device="cuda")
        x, y = t(rng.uniform(30, 30 + W - 20, n)), t(rng.uniform(30, 30 + H - 20, n))
        th, v = t(rng.uniform(0, 2 * np.pi, n)), t(np.zeros(n))
        base = VFParams(width=W, height=H, radius=A["radius"], dt=A["dt"])
        pv = torch.tensor([1.0, 0.08, 1.0, 0.08, 1.0], dtype=torch.float64, device="cuda",
                          requires_grad=True)
        out = edge.rollout(pv, x, y, th, v, base, 20, checkpoint=10)
        edge.flocking_loss(out[0], out[1], out[2],
                           torch.tensor([700.0, 700.0], device="cuda")).backward()
    torch.cuda.synchronize()
    print(json.dumps({"profile_workload": which, "ok": True}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-forage", action="store_true")
    ap.add_argument("--min-device-s", type=float, default=1.0,
                    help="repeat the timed K-step sequence until this much step time")
    ap.add_argument("--max-repeats", type=int, default=2000)
    ap.add_argument("--profile-workload",
                    choices=["headline", "batched", "batched_torus", "forage",
                             "forage_collide", "edge"],
                    help="run a few eager steps of one leg's workload and exit (for ncu)")
    args = ap.parse_args()
    if args.profile_workload:
        profile_workload(args.profile_workload)
        return
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        run_reference(args, rank, world)       # rank 0 only; no process group needed
        return
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl")
    try:
        run_gb300(args, rank, world)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
