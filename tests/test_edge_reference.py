"""CPU checks of the FP64 reference of the continuum edge form (tests/_edge_ref.py), which the
GPU adjoint is compared against: its integrals agree with a brute-force sampling of the covered
set on the circle, and its autograd gradients agree with central finite differences."""
import math

import numpy as np
import pytest
import torch

import _edge_ref as ER


def brute_integrals(x, y, th, R, samples=2_000_000):
    """Covered set sampled on a fine grid of the circle; blob integrals by the midpoint rule,
    edge sums over the sampled transitions."""
    n = len(x)
    phi = -math.pi + (np.arange(samples) + 0.5) * (2 * math.pi / samples)
    out = []
    for i in range(n):
        cov = np.zeros(samples, bool)
        for j in range(n):
            if j == i:
                continue
            dx, dy = x[j] - x[i], y[j] - y[i]
            if dx == 0 and dy == 0:
                continue
            b = math.atan2(-dy, dx) - th[i]
            a = math.atan(R / math.hypot(dx, dy))
            diff = (phi - b + math.pi) % (2 * math.pi) - math.pi
            cov |= np.abs(diff) <= a
        w = 2 * math.pi / samples
        bc = -np.sum(np.cos(phi[cov])) * w
        bs = -np.sum(np.sin(phi[cov])) * w
        trans = cov != np.roll(cov, 1)          # boundary between sample k-1 and k
        edge_phi = phi[trans] - 0.5 * w
        ec = np.sum(np.cos(edge_phi))
        es = np.sum(np.sin(edge_phi))
        out.append((bc, bs, ec, es))
    return np.array(out)


@pytest.mark.parametrize("seed,n,W,R", [(0, 8, 200.0, 10.0), (1, 12, 80.0, 10.0),
                                        (2, 6, 40.0, 12.0), (3, 10, 400.0, 5.0)])
def test_reference_integrals_vs_brute_force(seed, n, W, R):
    rng = np.random.default_rng(seed)
    x = rng.uniform(0, W, n)
    y = rng.uniform(0, W, n)
    th = rng.uniform(0, 2 * math.pi, n)
    t = lambda a: torch.tensor(a, dtype=torch.float64)
    bc, bs, ec, es = ER.edge_integrals(t(x), t(y), t(th), R)
    ref = brute_integrals(x, y, th, R)
    got = torch.stack([bc, bs, ec, es], 1).numpy()
    assert np.allclose(got[:, :2], ref[:, :2], atol=2e-5)
    assert np.allclose(got[:, 2:], ref[:, 2:], atol=1e-4)


def test_reference_gradients_vs_central_fd():
    rng = np.random.default_rng(5)
    n, steps, R, dt = 12, 12, 10.0, 0.1
    W = 300.0
    bounds = (30.0, 30.0 + W, 30.0, 30.0 + W)
    x = torch.tensor(rng.uniform(60, 300, n), dtype=torch.float64)
    y = torch.tensor(rng.uniform(60, 300, n), dtype=torch.float64)
    th = torch.tensor(rng.uniform(0, 2 * math.pi, n), dtype=torch.float64)
    v = torch.zeros(n, dtype=torch.float64)
    target = torch.tensor([150.0, 170.0], dtype=torch.float64)
    base = {"gam": 0.1}
    p0 = torch.tensor([1.0, 0.08, 1.0, 0.08, 1.0], dtype=torch.float64, requires_grad=True)
    out = ER.rollout(p0, x, y, th, v, base, R, dt, bounds, steps)
    L = ER.loss(*out[:3], target)
    (g,) = torch.autograd.grad(L, p0)
    h = 1e-4
    for k in range(5):
        e = torch.zeros(5, dtype=torch.float64)
        e[k] = h
        with torch.no_grad():
            lp = ER.loss(*ER.rollout(p0 + e, x, y, th, v, base, R, dt, bounds, steps)[:3], target)
            lm = ER.loss(*ER.rollout(p0 - e, x, y, th, v, base, R, dt, bounds, steps)[:3], target)
        fd = float((lp - lm) / (2 * h))
        assert abs(fd - float(g[k])) <= 1e-6 * max(1.0, abs(fd)), (k, fd, float(g[k]))
