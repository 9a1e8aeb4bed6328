"""GPU tests of the differentiable edge form (abm_vpf_edge_fwd / abm_vpf_edge_bwd, and the
torch.autograd.Function in abm_gb300.edge):

* forward integrals against the FP64 reference (tests/_edge_ref.py);
* the pixel VPF at high Rv converges to the edge form (the pixel path is the arbiter);
* adjoint gradients (alp0, alp1, beta0, beta1, v0 and the initial state) against FP64 autograd
  and against FP64 central finite differences at h = 1e-4: within 1e-4 relative;
* at the full differentiable workload (N=256, 200 steps, checkpoint every 20) the float32
  kernels segment by segment: each 20-step segment's gradient from the float32 rollout's own
  checkpoint against FP64 autograd of the same segment from the same state, and 5-step
  sub-segments against FD at h = 1e-4 wherever no arc event lies within the perturbation.

The edge form is piecewise smooth: arc merges and splits are jumps of the edge terms.  Central
FD at h is a derivative only if no event lies within +-h; this is detected by comparing FD(h)
with FD(h/2) (a jump J shows as J/2h, doubling when h halves): FD(h) counts as a derivative
when the two differ by at most half the 1e-4 bar (FD_CONSISTENT).
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
    # relative to each integral's scale over the swarm (single values cancel towards zero)
    rel = np.abs(got - ref) / np.maximum(np.abs(ref).max(axis=0), 1e-12)
    assert rel.max() <= 1e-4, rel.max(axis=0)


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


FD_CONSISTENT = 5e-5   # |FD(h) - FD(h/2)| / scale at which FD(h) is a derivative


def _fd(f, p0, k, h):
    e = torch.zeros(5, dtype=torch.float64, device=p0.device)
    e[k] = h
    with torch.no_grad():
        return (f(p0 + e) - f(p0 - e)) / (2 * h)


@pytest.mark.parametrize("seed,n,W,steps,ckpt,dtype", [
    (3, 32, 300.0, 40, 10, torch.float32),
    (4, 64, 600.0, 60, 20, torch.float64),
    (6, 48, 250.0, 50, 20, torch.float64),
])
def test_adjoint_vs_fp64_autograd(seed, n, W, steps, ckpt, dtype):
    """float32 where its rounding does not move the rollout (short horizon, small swarm), and
    the double-precision kernels otherwise: parameter and initial-state gradients within 1e-4
    of FP64 autograd."""
    x, y, th, v = _swarm(seed, n, W)
    base = _base(W)
    target = (0.4 * W, 0.55 * W)
    pv = [1.0, 0.08, 1.0, 0.08, 1.0]
    Lg, gg = _grad_gpu(x, y, th, v, base, steps, ckpt, target, pv, dtype)
    Lr, gr, p, init, bounds = _grad_fp64(x, y, th, v, base, steps, target, pv)
    assert abs(Lg - Lr) <= 1e-5 * max(1.0, abs(Lr))
    for k, (a, b) in enumerate(zip(gg, gr)):
        assert _rel(a, b) <= 1e-4, (k, _rel(a, b))


def test_adjoint_float32_vs_central_fd():
    """FP64 central finite differences at h = 1e-4 of the five parameters, on a horizon where
    no arc event lies within the perturbation (FD(h) = FD(h/2) for every component): the
    float32 adjoint within 1e-4 (relative to the gradient's scale) of all five."""
    seed, n, W, steps = 3, 32, 300.0, 40
    x, y, th, v = _swarm(seed, n, W)
    base = _base(W)
    target = (0.4 * W, 0.55 * W)
    pv = [1.0, 0.08, 1.0, 0.08, 1.0]
    _, gg = _grad_gpu(x, y, th, v, base, steps, 10, target, pv, torch.float32)
    _, gr, p, init, bounds = _grad_fp64(x, y, th, v, base, steps, target, pv)
    f = lambda q: float(ER.loss(*ER.rollout(q, *[t.detach() for t in init], {"gam": base.gam},
                                           base.radius, base.dt, bounds, steps)[:3],
                                torch.tensor(target, dtype=torch.float64)))
    scale = np.max(np.abs(gr[0]))
    p0 = p.detach()
    for k in range(5):
        a, b = _fd(f, p0, k, 1e-4), _fd(f, p0, k, 5e-5)
        assert abs(a - b) <= FD_CONSISTENT * scale, ("event within h", k, a, b)
        assert abs(gg[0][k] - a) <= 1e-4 * scale, (k, gg[0][k], a)


def test_adjoint_float32_segments_full_size():
    """The differentiable workload (N=256, radius 10, 1500x1500, 200 steps at dt = 0.1,
    checkpoint every 20) with the float32 kernels, segment by segment, so that the comparison
    does not depend on float32 and FP64 whole trajectories taking the same arc events: the
    float32 rollout's checkpoint states S_0 .. S_9 (every 20 steps); for each segment, the
    float32 kernels' gradient of the loss at the segment's end w.r.t. the five parameters and
    the segment's start state (x, y, theta, v) against FP64 autograd of the same 20 steps from
    the same S_s: within 1e-4 relative.  Then 5-step sub-segments from each S_s against FP64
    central FD at h = 1e-4 of all five parameters, accepted where no arc event lies within
    +-h (FD(h) = FD(h/2) to FD_CONSISTENT); every parameter must be checked on at least half
    of the segments."""
    from abm_gb300 import edge
    n, W, steps, K = 256, 1500.0, 200, 20
    x, y, th, _ = _swarm(11, n, W)
    v = np.zeros(n, np.float32)
    base = _base(W)
    target = (700.0, 800.0)
    pv = [1.0, 0.08, 1.0, 0.08, 1.0]
    dev = torch.device("cuda")
    p32 = torch.tensor(pv, dtype=torch.float64, device=dev)
    state = [torch.tensor(a, dtype=torch.float32, device=dev) for a in (x, y, th, v)]
    starts = []
    with torch.no_grad():
        for s in range(steps // K):
            starts.append([t.clone() for t in state])
            state = list(edge.rollout(p32, *state, base=base, steps=K, checkpoint=K))
    bounds = (base.window_pad, base.window_pad + W, base.window_pad, base.window_pad + W)
    tgt64 = torch.tensor(target, dtype=torch.float64, device=dev)

    def gpu_grad(S, L):
        p = torch.tensor(pv, dtype=torch.float64, device=dev, requires_grad=True)
        init = [t.clone().requires_grad_(True) for t in S]
        out = edge.rollout(p, *init, base=base, steps=L, checkpoint=K)
        loss = edge.flocking_loss(out[0], out[1], out[2],
                                  torch.tensor(target, dtype=torch.float32, device=dev))
        return [g.detach().cpu().numpy().astype(np.float64)
                for g in torch.autograd.grad(loss, [p] + init)]

    def ref_grad(S, L):
        p = torch.tensor(pv, dtype=torch.float64, device=dev, requires_grad=True)
        init = [t.detach().to(torch.float64).requires_grad_(True) for t in S]
        out = ER.rollout(p, *init, {"gam": base.gam}, base.radius, base.dt, bounds, L)
        loss = ER.loss(*out[:3], tgt64)
        return [g.detach().cpu().numpy() for g in torch.autograd.grad(loss, [p] + init)]

    worst = np.zeros(5)
    for s, S in enumerate(starts):
        gg, gr = gpu_grad(S, K), ref_grad(S, K)
        for k in range(5):
            r = _rel(gg[k], gr[k])
            worst[k] = max(worst[k], r)
            assert r <= 1e-4, ("segment", s, "component", k, r)
    print("segment VJP worst relative error (params, x, y, theta, v):", worst)

    checked = np.zeros(5, int)
    for s, S in enumerate(starts):
        L = 5
        gg = gpu_grad(S, L)
        S64 = [t.to(torch.float64) for t in S]
        f = lambda q: float(ER.loss(*ER.rollout(q, *S64, {"gam": base.gam}, base.radius,
                                               base.dt, bounds, L)[:3], tgt64))
        p0 = torch.tensor(pv, dtype=torch.float64, device=dev)
        scale = np.max(np.abs(gg[0]))
        for k in range(5):
            a, b = _fd(f, p0, k, 1e-4), _fd(f, p0, k, 5e-5)
            if abs(a - b) > FD_CONSISTENT * scale:
                continue                      # an arc event lies within +-h
            checked[k] += 1
            assert abs(gg[0][k] - a) <= 1e-4 * scale, ("segment", s, k, gg[0][k], a)
    print("FD (h = 1e-4) checks per parameter (alp0, alp1, bet0, bet1, v0):", checked)
    assert np.all(checked >= len(starts) // 2), checked


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
    for k in range(5):   # parameters, x, y, theta, v
        assert _rel(gg[k], gr[k]) <= 1e-4, (k, _rel(gg[k], gr[k]))
