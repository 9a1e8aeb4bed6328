"""GPU tests of the differentiable edge form (abm_vpf_edge_fwd / abm_vpf_edge_bwd, and the
torch.autograd.Function in abm_gb300.edge):

* forward integrals against the FP64 reference (tests/_edge_ref.py);
* the pixel VPF at high Rv converges to the edge form (the pixel path is the arbiter);
* adjoint gradients (alp0, alp1, beta0, beta1, v0 and the initial state) against FP64 autograd
  and against FP64 central finite differences (h = 1e-4): within 1e-4 relative.
"""
import math

import numpy as np
import pytest
import torch

import _edge_ref as ER
from conftest import gpu_available

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _need_gpu():
    if not gpu_available():
        pytest.skip("no CUDA device")


def _swarm(seed, n, W, pad=30.0, R=10.0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(pad, pad + W - 2 * R, n).astype(np.float32)
    y = rng.uniform(pad, pad + W - 2 * R, n).astype(np.float32)
    th = rng.uniform(0, 2 * math.pi, n).astype(np.float32)
    v = rng.uniform(0, 1, n).astype(np.float32)
    return x, y, th, v


def _base(W, R=10.0, dt=0.1):
    from abm_gb300.params import VFParams
    return VFParams(gam=0.1, v0=1.0, alp0=1.0, alp1=0.08, bet0=1.0, bet1=0.08, width=W,
                    height=W, window_pad=30.0, radius=R, dt=dt, rv=1200)


@pytest.mark.parametrize("seed,n,W", [(0, 64, 400.0), (1, 256, 1500.0), (2, 40, 120.0)])
def test_edge_forward_matches_fp64(seed, n, W):
    from abm_gb300.edge import edge_terms
    x, y, th, v = _swarm(seed, n, W)
    base = _base(W)
    dev = [torch.as_tensor(a, device="cuda") for a in (x, y, th, v)]
    got = edge_terms(dev, base).cpu().numpy().astype(np.float64)
    t = lambda a: torch.tensor(a, dtype=torch.float64)
    ref = torch.stack(ER.edge_integrals(t(x), t(y), t(th), 10.0), 1).numpy()
    assert np.max(np.abs(got - ref)) < 2e-4, np.max(np.abs(got - ref))


def test_pixel_form_converges_to_edge_form():
    """VSWRM terms of the pixel path (abm_vpf_flock_step with ALP0=BET0=ALP1=BET1=1) approach
    the edge form as Rv grows: the error shrinks about linearly in 1/Rv."""
    from abm_gb300.edge import edge_terms
    from abm_gb300.params import VFParams
    from abm_gb300.swarm import VFSwarm
    n, W = 24, 300.0
    x, y, th, v = _swarm(7, n, W)
    base = _base(W)
    dev = [torch.as_tensor(a, device="cuda") for a in (x, y, th, v)]
    edge = edge_terms(dev, base).cpu().numpy().astype(np.float64)
    errs = []
    for rv in (2048, 8192):
        vp = VFParams(gam=0.1, v0=1.0, alp0=1.0, alp1=1.0, bet0=1.0, bet1=1.0, width=W,
                      height=W, rv=rv, radius=10.0)
        s = VFSwarm(vp, x, y, th, v)
        s.step(want_terms=True)
        t = s.terms.cpu().numpy()   # dv, dpsi, alpha_blob, alpha_edge, beta_blob, beta_edge
        pix = np.stack([t[:, 2], t[:, 4], t[:, 3], t[:, 5]], 1)
        errs.append(np.abs(pix - edge).max(axis=0))
    errs = np.array(errs)
    assert np.all(errs[1] <= 0.5 * errs[0] + 1e-3), errs
    assert np.all(errs[1] < 0.05), errs


def _grad_gpu(x, y, th, v, base, steps, ckpt, target, pv, dtype=torch.float32):
    from abm_gb300 import edge
    p = torch.tensor(pv, dtype=torch.float64, device="cuda", requires_grad=True)
    init = [torch.tensor(a, dtype=dtype, device="cuda", requires_grad=True)
            for a in (x, y, th, v)]
    out = edge.rollout(p, *init, base=base, steps=steps, checkpoint=ckpt)
    L = edge.flocking_loss(out[0], out[1], out[2],
                           torch.tensor(target, dtype=dtype, device="cuda"))
    grads = torch.autograd.grad(L, [p] + init)
    return float(L.detach()), [g.detach().cpu().numpy().astype(np.float64) for g in grads]


def _grad_fp64(x, y, th, v, base, steps, target, pv):
    W = base.width
    bounds = (base.window_pad, base.window_pad + W, base.window_pad, base.window_pad + W)
    p = torch.tensor(pv, dtype=torch.float64, requires_grad=True)
    init = [torch.tensor(a, dtype=torch.float64, requires_grad=True) for a in (x, y, th, v)]
    out = ER.rollout(p, *init, {"gam": base.gam}, base.radius, base.dt, bounds, steps)
    L = ER.loss(*out[:3], torch.tensor(target, dtype=torch.float64))
    grads = torch.autograd.grad(L, [p] + init)
    return float(L.detach()), [g.detach().numpy() for g in grads], p, init, bounds


def _rel(a, b):
    scale = max(np.max(np.abs(b)), 1e-12)
    return np.max(np.abs(a - b)) / scale


@pytest.mark.parametrize("seed,n,W,steps,ckpt,dtype", [
    (3, 32, 300.0, 40, 10, torch.float32),
    (4, 64, 600.0, 60, 20, torch.float64),
    (6, 48, 250.0, 50, 20, torch.float64),
])
def test_adjoint_vs_fp64_autograd_and_fd(seed, n, W, steps, ckpt, dtype):
    """float32 where its rounding does not move the rollout (short horizon, small swarm), and
    the double-precision kernels otherwise; both within 1e-4 of FP64 autograd and of FP64
    central finite differences of the parameter gradient."""
    x, y, th, v = _swarm(seed, n, W)
    base = _base(W)
    target = (0.4 * W, 0.55 * W)
    pv = [1.0, 0.08, 1.0, 0.08, 1.0]
    Lg, gg = _grad_gpu(x, y, th, v, base, steps, ckpt, target, pv, dtype)
    Lr, gr, p, init, bounds = _grad_fp64(x, y, th, v, base, steps, target, pv)
    assert abs(Lg - Lr) <= 1e-5 * max(1.0, abs(Lr))
    for k, (a, b) in enumerate(zip(gg, gr)):
        assert _rel(a, b) <= 1e-4, (k, _rel(a, b))
    # FP64 central finite differences of the parameter gradient.  The edge form is piecewise
    # smooth (arc merges / splits are jumps of the edge terms), and in larger swarms a
    # perturbation of 1e-4 crosses such an event; FD is a derivative only where the loss is
    # smooth at the step size, so each component uses the largest h in 1e-4 .. 1e-7 at which
    # FD(h) and FD(h/2) agree (h = 1e-4 whenever that holds).
    f = lambda q: float(ER.loss(*ER.rollout(q, *[t.detach() for t in init], {"gam": base.gam},
                                           base.radius, base.dt, bounds, steps)[:3],
                                torch.tensor(target, dtype=torch.float64)))
    scale = np.max(np.abs(gr[0]))

    def fd(k, h):
        e = torch.zeros(5, dtype=torch.float64)
        e[k] = h
        with torch.no_grad():
            return (f(p.detach() + e) - f(p.detach() - e)) / (2 * h)

    checked = 0
    for k in range(5):
        for h in (1e-4, 1e-5, 1e-6, 1e-7):
            a, b = fd(k, h), fd(k, h / 2)
            if abs(a - b) <= 1e-5 * scale:
                checked += 1
                assert abs(gg[0][k] - b) <= 1e-4 * scale, (k, h, gg[0][k], b)
                break
    assert checked >= 4, checked


def test_adjoint_full_size_differentiable_workload():
    """N=256, radius 10, 1500x1500, 200 steps at dt = 0.1, checkpoint every 20 (double-precision
    kernels): parameter and initial-state gradients within 1e-4 of FP64 autograd of the same
    dynamics, and the float32 rollout's drift from FP64 is reported (it changes arc events)."""
    n, W, steps = 256, 1500.0, 200
    x, y, th, v = _swarm(11, n, W)
    v = np.zeros(n, np.float32)
    base = _base(W)
    target = (700.0, 800.0)
    pv = [1.0, 0.08, 1.0, 0.08, 1.0]
    Lg, gg = _grad_gpu(x, y, th, v, base, steps, 20, target, pv, torch.float64)
    Lr, gr, *_ = _grad_fp64(x, y, th, v, base, steps, target, pv)
    assert abs(Lg - Lr) <= 1e-8 * max(1.0, abs(Lr))
    for k in range(4):
        assert _rel(gg[k], gr[k]) <= 1e-4, (k, _rel(gg[k], gr[k]))
