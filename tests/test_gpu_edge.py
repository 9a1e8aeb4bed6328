"""GPU tests of the differentiable edge form (abm_vpf_edge_fwd / abm_vpf_edge_bwd, and the
torch.autograd.Function in abm_gb300.edge):

* forward integrals against the FP64 reference (tests/_edge_ref.py);
* the pixel VPF at high Rv converges to the edge form (the pixel path is the arbiter);
* adjoint gradients (alp0, alp1, beta0, beta1, v0 and the initial state) against FP64 autograd
  and against FP64 central finite differences at h = 1e-4: within 1e-4 relative;
* at the full differentiable workload (N=256, 200 steps, checkpoint every 20): the float32
  kernels' one-step adjoints from the float32 rollout's checkpoint states against FP64
  autograd of the same step, agent by agent, away from arc events; the FP64 reference against
  FD at h = 1e-4 on 5-step sub-segments wherever no arc event lies within the perturbation;
  the double-precision kernels against FP64 autograd over all 200 steps.

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


def _full_size_workload():
    n, W = 256, 1500.0
    x, y, th, _ = _swarm(11, n, W)
    return x, y, th, np.zeros(n, np.float32), _base(W), (700.0, 800.0)


def _float32_checkpoints(x, y, th, v, base, pv, steps=200, K=20):
    """The float32 rollout's states every K steps (its checkpoints)."""
    from abm_gb300 import edge
    dev = torch.device("cuda")
    p = torch.tensor(pv, dtype=torch.float64, device=dev)
    state = [torch.tensor(a, dtype=torch.float32, device=dev) for a in (x, y, th, v)]
    starts = []
    with torch.no_grad():
        for _ in range(steps // K):
            starts.append([t.clone() for t in state])
            state = list(edge.rollout(p, *state, base=base, steps=K, checkpoint=K))
    return starts


def test_adjoint_float32_steps_full_size():
    """The differentiable workload (N=256, radius 10, 1500x1500, dt = 0.1) with the float32
    kernels: at each of the float32 rollout's checkpoint states (every 20 of 200 steps), the
    adjoint of one step for a cotangent on one agent's outputs at a time (x, y, theta, v),
    against FP64 autograd of the same step from the same state: the state and parameter
    gradients within 1e-4 relative for every agent whose arcs lie at least 1e-5 rad from an
    event of the edge form (and whose new centre is at least 1e-3 px from a wall).  Near an
    event the step is not differentiable at float32 resolution (float32 and FP64 may take
    either side); those agents are counted and must be a small minority.  Over whole 20-step
    segments float32 rounding moves such events, so segment gradients are compared against
    FP64 only through the double-precision kernels (test_adjoint_full_size_...)."""
    import ctypes
    from abm_gb300 import _lib, edge
    lib = _lib.load()
    x, y, th, v, base, _ = _full_size_workload()
    pv = [1.0, 0.08, 1.0, 0.08, 1.0]
    n, W = len(x), base.width
    dev = torch.device("cuda")
    bounds = (base.window_pad, base.window_pad + W, base.window_pad, base.window_pad + W)
    cp = edge._cparams(base, pv)
    rng = np.random.default_rng(5)
    checked = near = 0
    worst = np.zeros(2)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for S in _float32_checkpoints(x, y, th, v, base, pv):
        cot = rng.normal(size=(n, 4))
        # float32 kernels: one adjoint launch per agent's cotangent
        gout = [torch.zeros(n, dtype=torch.float32, device=dev) for _ in range(4)]
        gin = [torch.zeros(n, dtype=torch.float32, device=dev) for _ in range(4)]
        gp = torch.zeros(5, dtype=torch.float64, device=dev)
        s_in, s_go, s_gi = edge._state(S), edge._state(gout), edge._state(gin)
        got_state, got_par = np.zeros((n, 4, n)), np.zeros((n, 5))
        for i in range(n):
            for r in range(4):
                gout[r].zero_()
                gout[r][i] = float(cot[i, r])
            gp.zero_()
            _lib.check(lib.abm_vpf_edge_bwd(ctypes.byref(s_in), ctypes.byref(s_go),
                                            ctypes.byref(s_gi), _lib.dptr(gp), n,
                                            ctypes.byref(cp), 0, stream))
            got_state[i] = torch.stack(gin).cpu().numpy()
            got_par[i] = gp.cpu().numpy()
        # FP64 autograd of the same step from the same state
        p = torch.tensor(pv, dtype=torch.float64, device=dev, requires_grad=True)
        st = [t.detach().to(torch.float64).requires_grad_(True) for t in S]
        prm = {"gam": base.gam, "alp0": p[0], "alp1": p[1], "bet0": p[2], "bet1": p[3],
               "v0": p[4]}
        out = ER.edge_step(*st, prm, base.radius, base.dt, bounds)
        with torch.no_grad():
            marg = ER.event_margins(*[t.detach() for t in st[:3]], base.radius, bounds,
                                    v=st[3].detach(), p={k: float(prm[k]) for k in prm},
                                    dt=base.dt)
        ok = ((marg["arc"] >= 1e-5) & (marg["wall"] >= 1e-3)).cpu().numpy()
        ct = torch.tensor(cot, dtype=torch.float64, device=dev)
        for i in range(n):
            if not ok[i]:
                near += 1
                continue
            sel = sum(out[r][i] * ct[i, r] for r in range(4))
            g = torch.autograd.grad(sel, st + [p], retain_graph=True, allow_unused=True)
            want_state = np.stack([(torch.zeros(n, dtype=torch.float64, device=dev)
                                    if gg is None else gg).cpu().numpy() for gg in g[:4]])
            want_par = g[4].cpu().numpy()
            rs = _rel(got_state[i], want_state)
            rp = _rel(got_par[i], want_par)
            worst = np.maximum(worst, [rs, rp])
            assert rs <= 1e-4 and rp <= 1e-4, ("agent", i, rs, rp)
            checked += 1
    print(f"one-step float32 adjoints: {checked} agent-steps checked, worst relative error "
          f"state {worst[0]:.1e}, parameters {worst[1]:.1e}; {near} within 1e-5 rad of an arc "
          "event or 1e-3 px of a wall")
    assert near <= 0.2 * (checked + near), (checked, near)


def test_full_size_fd_validates_fp64_reference():
    """FP64 central finite differences at h = 1e-4 of the five parameters against FP64 autograd
    at the differentiable workload (N=256), from each of the float32 rollout's checkpoints, on
    the longest sub-segment of 5, 3, 2 or 1 steps on which no arc event lies within +-h
    (FD(h) = FD(h/2) to FD_CONSISTENT).  Over one step the arcs are those of the step's input
    state and the increments are linear in the parameters, so such a sub-segment always exists:
    every parameter is checked at every checkpoint."""
    x, y, th, v, base, target = _full_size_workload()
    pv = [1.0, 0.08, 1.0, 0.08, 1.0]
    W = base.width
    dev = torch.device("cuda")
    bounds = (base.window_pad, base.window_pad + W, base.window_pad, base.window_pad + W)
    tgt64 = torch.tensor(target, dtype=torch.float64, device=dev)
    starts = _float32_checkpoints(x, y, th, v, base, pv)
    lengths = np.zeros((len(starts), 5), int)
    for s, S in enumerate(starts):
        S64 = [t.to(torch.float64) for t in S]
        for L in (5, 3, 2, 1):
            p = torch.tensor(pv, dtype=torch.float64, device=dev, requires_grad=True)
            out = ER.rollout(p, *S64, {"gam": base.gam}, base.radius, base.dt, bounds, L)
            g = torch.autograd.grad(ER.loss(*out[:3], tgt64), p)[0].cpu().numpy()
            f = lambda q: float(ER.loss(*ER.rollout(q, *S64, {"gam": base.gam}, base.radius,
                                                   base.dt, bounds, L)[:3], tgt64))
            p0 = p.detach()
            scale = np.max(np.abs(g))
            for k in np.where(lengths[s] == 0)[0]:
                a, b = _fd(f, p0, k, 1e-4), _fd(f, p0, k, 5e-5)
                if abs(a - b) > FD_CONSISTENT * scale:
                    continue                      # an arc event lies within +-h
                lengths[s, k] = L
                assert abs(g[k] - a) <= 1e-4 * scale, ("checkpoint", s, "steps", L, k, g[k], a)
            if np.all(lengths[s] > 0):
                break
    print("FD (h = 1e-4) sub-segment lengths, checkpoint x parameter (alp0, alp1, bet0, bet1, "
          "v0):", lengths.tolist())
    assert np.all(lengths > 0), lengths


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
