"""Long runs: ensemble statistics of the snapshot (Jacobi) dynamics against whole runs of the
reference's own sequential loop.

tests/golden/vf_ensemble.npz (make_vf_ensemble.py) holds 32 runs of the plain flocking
workload (N=10, 500 x 500 walls, Rv=1200, 1000 steps) played by the reference's VFAgent in its
group order (vf_ensemble_torus.npz: the same on the torus), each agent seeing the agents before it already moved.  Single trajectories
diverge from any other update order or precision, so the comparison is the run mean of the
time-averaged polarisation over the second half (data_loader.py:1818-1824), within four
combined standard errors.
"""
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN, gpu_available

T0 = 500


def _ref(name="vf_ensemble.npz"):
    z = np.load(os.path.join(GOLDEN, name))
    p = {k: float(v) for k, v in zip(oracle.P_FIELDS, z["params"])}
    init = {k: z["init_" + k] for k in ("x", "y", "theta")}
    return z, p, init


def _polarisation(theta):
    th = np.asarray(theta, np.float64)
    return np.hypot(np.cos(th).sum(axis=-1), np.sin(th).sum(axis=-1)) / th.shape[-1]


def _close(a, b):
    se = np.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
    assert abs(a.mean() - b.mean()) <= 4 * se, (a.mean(), b.mean(), se)


@pytest.mark.parametrize("name", ["vf_ensemble.npz", "vf_ensemble_torus.npz"])
def test_oracle_snapshot_ensemble_matches_reference_runs(name):
    """The oracle's snapshot step (the GPU's update order, FP64) from the same initial
    states, in the walls arena and on the torus."""
    z, p, init = _ref(name)
    ref = z["pol"][:, T0:].mean(axis=1)
    runs, T = z["pol"].shape
    res = []
    for r in range(runs):
        st = {k: init[k][r].copy() for k in init}
        st["v"] = np.zeros_like(st["x"])
        acc = []
        for t in range(T):
            st = oracle.vf_step(st, p, want_vpf=False, want_terms=False)
            if t >= T0:
                acc.append(_polarisation(st["theta"]))
        res.append(np.mean(acc))
    _close(np.array(res), ref)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["vf_ensemble.npz", "vf_ensemble_torus.npz"])
def test_gpu_ensemble_matches_reference_runs(name):
    """256 GPU runs (the reference's 32 initial states and 224 more drawn the same way) in one
    batched sweep with the on-device polarisation series, in the walls arena and on the
    torus."""
    if not gpu_available():
        pytest.skip("no CUDA device")
    from abm_gb300.batched import BatchedSweep
    from abm_gb300.params import VFParams
    z, p, init = _ref(name)
    runs, T = z["pol"].shape
    n = init["x"].shape[1]
    insts = [{"x": init["x"][r].astype(np.float32), "y": init["y"][r].astype(np.float32),
              "theta": init["theta"][r].astype(np.float32)} for r in range(runs)]
    pad, R, W = p["window_pad"], p["radius"], p["width"]
    for seed in range(1000, 1224):
        rng = np.random.default_rng(seed)
        insts.append({"x": rng.uniform(pad - R, pad + W - R, n).astype(np.float32),
                      "y": rng.uniform(pad - R, pad + W - R, n).astype(np.float32),
                      "theta": rng.uniform(0, 2 * np.pi, n).astype(np.float32)})
    vp = VFParams(alp1=p["alp1"], bet1=p["bet1"], width=W, height=p["height"], rv=int(p["rv"]),
                  radius=R, boundary="infinite" if p["boundary"] else "walls")
    sweep = BatchedSweep(vp, insts)
    sweep.track_polarisation(T)
    sweep.run(T, chunk=100)
    pol = sweep.polarisation()
    assert pol.shape == (len(insts), T)
    _close(pol[:, T0:].mean(axis=1), z["pol"][:, T0:].mean(axis=1))
