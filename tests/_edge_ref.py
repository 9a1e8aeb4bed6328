"""FP64 torch-autograd reference of the continuum edge form (test infrastructure).

The same discrete dynamics as abm_vpf_edge_fwd (abm_gb300/csrc/vpf_edge.cu), written with
vectorised torch ops so autograd gives exact FP64 gradients: per focal agent the arcs
[b_j - a_j, b_j + a_j] are sorted by lower end, merged with a running maximum of the upper
ends, the seam is closed by folding the leading arcs into the last one, and the integrals are
sums of sin/cos of the merged arc ends.
"""
import math

import torch

TWO_PI = 2 * math.pi
BIG = 1e30


def edge_integrals(x, y, th, R, use_asin=False):
    n = x.shape[0]
    dx = x[None, :] - x[:, None]          # [i, j] = x_j - x_i
    dy = y[None, :] - y[:, None]
    eye = torch.eye(n, dtype=torch.bool, device=x.device)
    valid = ~eye & ((dx != 0) | (dy != 0))
    dxs = torch.where(valid, dx, torch.ones_like(dx))
    dys = torch.where(valid, dy, torch.zeros_like(dy))
    b = torch.atan2(-dys, dxs) - th[:, None]
    b = b - TWO_PI * torch.round(b / TWO_PI)
    d = torch.sqrt(dxs * dxs + dys * dys)
    if use_asin:
        a = torch.where(d > R, torch.asin(torch.clamp(R / d, max=1.0)),
                        torch.full_like(d, math.pi / 2))
    else:
        a = torch.atan(R / d)
    lo = b - a
    lo = torch.where(lo < -math.pi, lo + TWO_PI, lo)
    up = lo + 2 * a
    lo = torch.where(valid, lo, torch.full_like(lo, BIG))
    up = torch.where(valid, up, torch.full_like(up, -BIG))
    lo_s, order = torch.sort(lo, dim=1)
    up_s = torch.gather(up, 1, order)
    pm = torch.cummax(up_s, dim=1).values
    vmask = lo_s < BIG / 2
    prev = torch.cat([torch.full((n, 1), -BIG, dtype=x.dtype, device=x.device), pm[:, :-1]], 1)
    start = vmask & (lo_s > prev)
    tail = torch.ones((n, 1), dtype=torch.bool, device=x.device)
    end = vmask & (torch.cat([start[:, 1:], tail], 1) | torch.cat([~vmask[:, 1:], tail], 1))
    K = start.sum(1)
    ulast = pm[:, -1]
    fold_start = start & (lo_s + TWO_PI <= ulast[:, None])
    fold = fold_start.sum(1)
    srank = torch.cumsum(start.long(), 1) - 1
    erank = torch.cumsum(end.long(), 1) - 1
    full = (K > 0) & (fold >= K)
    keep_lo = start & (srank >= fold[:, None]) & ~full[:, None]
    last = end & (erank == (K - 1)[:, None])
    keep_hi = end & (erank >= fold[:, None]) & ~last & ~full[:, None]
    # upper end of the last arc, extended by the folded arcs
    prev_fold_end = end & (erank == (fold - 1)[:, None])
    u_prev = torch.where(prev_fold_end, pm + TWO_PI, torch.full_like(pm, -BIG)).max(1).values
    new_hi = torch.maximum(ulast, u_prev)
    has_last = (K > 0) & ~full
    z = torch.zeros((), dtype=x.dtype, device=x.device)
    sl, cl = torch.sin(lo_s), torch.cos(lo_s)
    su, cu = torch.sin(pm), torch.cos(pm)
    sn, cn = torch.sin(new_hi), torch.cos(new_hi)
    kl, kh = keep_lo.to(x.dtype), keep_hi.to(x.dtype)
    lo_term = lambda v: torch.where(keep_lo, v, z).sum(1)
    hi_term = lambda v: torch.where(keep_hi, v, z).sum(1)
    hl = has_last.to(x.dtype)
    bc = lo_term(sl) - hi_term(su) - hl * sn
    bs = -lo_term(cl) + hi_term(cu) + hl * cn
    ec = lo_term(cl) + hi_term(cu) + hl * cn
    es = lo_term(sl) + hi_term(su) + hl * sn
    del kl, kh
    return bc, bs, ec, es


def edge_step(x, y, th, v, p, R, dt, bounds, use_asin=False):
    """p: dict with gam, v0, alp0, alp1, bet0, bet1 (floats or 0-d tensors)."""
    bx0, bx1, by0, by1 = bounds
    bc, bs, ec, es = edge_integrals(x, y, th, R, use_asin)
    dv = p["gam"] * (p["v0"] - v) + p["alp0"] * bc + p["alp0"] * p["alp1"] * ec
    dpsi = p["bet0"] * bs + p["bet0"] * p["bet1"] * es
    t = th + dpsi * dt
    t = torch.where(t < 0, t + TWO_PI, t)
    t = torch.where(t > TWO_PI, t - TWO_PI, t)
    v1 = v + dv * dt
    x1 = x + v1 * torch.cos(t) * dt
    y1 = y - v1 * torch.sin(t) * dt
    cx, cy = x1 + R, y1 + R
    pi = math.pi

    def wrap(t):
        t = torch.where(t < 0, t + TWO_PI, t)
        return torch.where(t > TWO_PI, t - TWO_PI, t)

    m = cx < bx0
    x1 = torch.where(m, torch.full_like(x1, bx0 - R), x1)
    t = torch.where(m & (pi / 2 <= t) & (t < pi), t - pi / 2,
                    torch.where(m & (pi <= t) & (t <= 3 * pi / 2), t + pi / 2, t))
    t = torch.where(m, wrap(t), t)
    m = cx > bx1
    x1 = torch.where(m, torch.full_like(x1, bx1 - R - 1), x1)
    t = torch.where(m & (3 * pi / 2 <= t) & (t < TWO_PI), t - pi / 2,
                    torch.where(m & (0 <= t) & (t <= pi / 2), t + pi / 2, t))
    t = torch.where(m, wrap(t), t)
    m = cy < by0
    y1 = torch.where(m, torch.full_like(y1, by0 - R), y1)
    t = torch.where(m & (pi / 2 <= t) & (t <= pi), t + pi / 2,
                    torch.where(m & (0 <= t) & (t < pi / 2), t - pi / 2, t))
    t = torch.where(m, wrap(t), t)
    m = cy > by1
    y1 = torch.where(m, torch.full_like(y1, by1 - R - 1), y1)
    t = torch.where(m & (3 * pi / 2 <= t) & (t <= TWO_PI), t + pi / 2,
                    torch.where(m & (pi <= t) & (t < 3 * pi / 2), t - pi / 2, t))
    t = torch.where(m, wrap(t), t)
    return x1, y1, t, v1


def rollout(pvec, x, y, th, v, base, R, dt, bounds, steps, use_asin=False):
    """pvec = (alp0, alp1, bet0, bet1, v0) tensor; base: dict with gam."""
    p = {"gam": base["gam"], "alp0": pvec[0], "alp1": pvec[1], "bet0": pvec[2],
         "bet1": pvec[3], "v0": pvec[4]}
    for _ in range(steps):
        x, y, th, v = edge_step(x, y, th, v, p, R, dt, bounds, use_asin)
    return x, y, th, v


def loss(x, y, th, target, R=0.0):
    n = th.shape[0]
    pol = torch.sqrt(torch.cos(th).sum() ** 2 + torch.sin(th).sum() ** 2) / n
    mx, my = (x + R).mean(), (y + R).mean()
    return 1.0 - pol + ((mx - target[0]) ** 2 + (my - target[1]) ** 2) / 2.0


def event_margins(x, y, th, R, bounds, v=None, p=None, dt=0.1):
    """Per focal agent, the distance (radians) of its arc structure from the nearest event of
    the edge form -- an arc start decision (lower end vs the running maximum of the upper ends),
    the seam fold (lower end + 2 pi vs the last upper end), the wrap of a lower end at -pi or
    of a bearing at +-pi -- and, when the update's inputs v, p are given, the distance (pixels)
    of its new centre from a wall.  A gradient is a derivative of the step only away from these
    discontinuities."""
    n = x.shape[0]
    dx = x[None, :] - x[:, None]
    dy = y[None, :] - y[:, None]
    eye = torch.eye(n, dtype=torch.bool, device=x.device)
    valid = ~eye & ((dx != 0) | (dy != 0))
    dxs = torch.where(valid, dx, torch.ones_like(dx))
    dys = torch.where(valid, dy, torch.zeros_like(dy))
    b = torch.atan2(-dys, dxs) - th[:, None]
    b = b - TWO_PI * torch.round(b / TWO_PI)
    a = torch.atan(R / torch.sqrt(dxs * dxs + dys * dys))
    lo = b - a
    m_wrap = torch.where(valid, torch.minimum((lo + math.pi).abs(), (b.abs() - math.pi).abs()),
                         torch.full_like(lo, BIG))
    lo = torch.where(lo < -math.pi, lo + TWO_PI, lo)
    up = lo + 2 * a
    lo = torch.where(valid, lo, torch.full_like(lo, BIG))
    up = torch.where(valid, up, torch.full_like(up, -BIG))
    lo_s, order = torch.sort(lo, dim=1)
    up_s = torch.gather(up, 1, order)
    pm = torch.cummax(up_s, dim=1).values
    vmask = lo_s < BIG / 2
    gap = (lo_s[:, 1:] - pm[:, :-1]).abs()
    gap = torch.where(vmask[:, 1:], gap, torch.full_like(gap, BIG))
    ulast = pm.gather(1, (vmask.sum(1, keepdim=True) - 1).clamp(min=0))
    fold = torch.where(vmask, (lo_s + TWO_PI - ulast).abs(), torch.full_like(lo_s, BIG))
    m = torch.minimum(torch.minimum(gap.min(1).values, fold.min(1).values), m_wrap.min(1).values)
    out = {"arc": m}
    if v is not None and p is not None:
        x1, y1, _, _ = edge_step(x, y, th, v, p, R, dt, bounds)
        bx0, bx1, by0, by1 = bounds
        cx, cy = x1 + R, y1 + R
        out["wall"] = torch.stack([(cx - bx0).abs(), (cx - bx1).abs(), (cy - by0).abs(),
                                   (cy - by1).abs()], 1).min(1).values
    return out
