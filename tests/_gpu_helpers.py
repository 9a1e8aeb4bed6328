"""Helpers shared by the GPU parity tests (seeded swarms, the VPF check with its excuse mask)."""
import numpy as np

# Pixels of pairs whose edge angle lies within this many radians of a pixel / width decision
# boundary may differ from the reference (the FP32 / double-float decision against FP64).
NEAR_BAND = 1e-9


def f32(a):
    return np.asarray(a, dtype=np.float32).astype(np.float64)


def seeded_swarm(seed, n, W, H, pad=30.0, R=10.0, kappa=None, vmax=1.5):
    rng = np.random.default_rng(seed)
    x = f32(rng.uniform(pad - R, pad + W - R, n))
    y = f32(rng.uniform(pad - R, pad + H - R, n))
    if kappa is None:
        th = f32(rng.uniform(0, 2 * np.pi, n))
    else:
        th = f32(np.mod(rng.vonmises(rng.uniform(0, 2 * np.pi), kappa, n), 2 * np.pi))
    v = f32(rng.uniform(0, vmax, n))
    return {"x": x, "y": y, "theta": th, "v": v}


def check_vpf(gpu_vpf, want_vpf, excuse, near, what):
    """VPF bits exact, except pixels in the oracle's excuse mask: the pixels that pairs within
    NEAR_BAND rad of a decision boundary flip under their alternative decisions (never a whole
    row).  Returns (mismatched pixels, agents with a mismatch, near-boundary pairs); every
    agent with a mismatch has at least one near-boundary pair."""
    gpu_vpf = np.asarray(gpu_vpf, np.uint8)
    want_vpf = np.asarray(want_vpf, np.uint8)
    bad = gpu_vpf != want_vpf
    unexcused = bad & (np.asarray(excuse) == 0)
    if np.any(unexcused):
        rows = np.where(unexcused.any(axis=-1))[0] if unexcused.ndim > 1 else [0]
        r = rows[0]
        px = np.where(unexcused[r] if unexcused.ndim > 1 else unexcused)[0]
        raise AssertionError(f"{what}: VPF differs outside the excuse mask: agent {r}, "
                             f"pixels {px[:10]} ({int(unexcused.sum())} pixels in all)")
    bad_rows = int(bad.any(axis=-1).sum()) if bad.ndim > 1 else int(bad.any())
    n_near = int(np.sum(near))
    assert bad_rows <= n_near, (what, bad_rows, n_near)
    return int(bad.sum()), bad_rows, n_near
