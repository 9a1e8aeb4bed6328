"""The oracle's excuse mask (the only pixels a GPU VPF may differ in): for a pair whose bearing or
half visual angle lies within 1e-9 rad of a decision boundary, exactly the pixels on which its
alternative decisions differ -- checked on pairs placed on a pixel midpoint, on a width switch
and on the +-pi seam, and empty for pairs away from every boundary."""
import math

import numpy as np

import oracle

RV, R = 64, 10.0
POS = (100.0, 100.0)   # focal top-left; centre (110, 110), heading 0


def _place(ca, d):
    """Top-left of an object of radius R whose centre lies at bearing `ca` (math frame, left
    positive; screen y points down) and distance `d` from the focal centre."""
    cx, cy = POS[0] + R + d * math.cos(ca), POS[1] + R - d * math.sin(ca)
    return [cx - R, cy - R]


def _raw(rows):
    return rows[:, ::-1]   # projection_field's rows are flipped; back to raw pixel order


def test_pair_on_a_pixel_midpoint():
    phis = oracle.linspace(RV)
    k = 20
    m = 0.5 * (phis[k] + phis[k + 1])
    obj = [_place(m, 100.0)]      # half angle atan(0.1) = 1.015 px units: h = 1, far from 1 or 2
    rows, marg = oracle.projection_field((-math.pi, math.pi), RV, POS, R, 0.0, obj,
                                         return_margins=True)
    ex, near = oracle.projection_excuse((-math.pi, math.pi), RV, POS, R, 0.0, obj)
    assert marg[0] < 1e-9 and near[0]
    t = int(np.argmax(_raw(rows)[0])) + 1          # the row is [t - 1, t + 1)
    assert t in (k, k + 1)
    other = k + 1 if t == k else k
    # alternatives [t-1, t+1) and [other-1, other+1) differ in exactly two pixels
    want = sorted({t - 1, t} ^ {other - 1, other})
    assert sorted(np.where(_raw(ex)[0])[0].tolist()) == want


def test_pair_on_a_width_switch():
    phis = oracle.linspace(RV)
    t = 30
    unit = 2 * math.pi / RV
    d = R / math.tan(2 * unit)      # atan(R/d) = 2 units exactly: h flips between 1 and 2
    obj = [_place(phis[t], d)]
    rows, marg = oracle.projection_field((-math.pi, math.pi), RV, POS, R, 0.0, obj,
                                         return_margins=True)
    ex, near = oracle.projection_excuse((-math.pi, math.pi), RV, POS, R, 0.0, obj)
    assert marg[0] < 1e-9 and near[0]
    on = np.where(_raw(rows)[0])[0]
    h = len(on) // 2
    assert h in (1, 2) and on[0] == t - h
    # [t-1, t+1) vs [t-2, t+2): pixels t-2 and t+1
    assert sorted(np.where(_raw(ex)[0])[0].tolist()) == [t - 2, t + 1]


def test_pair_on_the_seam():
    """Exactly behind: the bearing is -pi (pixel 0) or just below pi (pixel Rv-1)."""
    obj = [_place(math.pi, 100.0)]
    rows, marg = oracle.projection_field((-math.pi, math.pi), RV, POS, R, 0.0, obj,
                                         return_margins=True)
    ex, near = oracle.projection_excuse((-math.pi, math.pi), RV, POS, R, 0.0, obj)
    assert marg[0] < 1e-9 and near[0]
    got = set(np.where(_raw(ex)[0])[0].tolist())
    assert got and got <= {0, 1, 2, RV - 3, RV - 2, RV - 1}


def test_far_from_boundaries_nothing_is_excused():
    rng = np.random.default_rng(5)
    objs = [_place(a, d) for a, d in zip(rng.uniform(-3, 3, 40), rng.uniform(25, 300, 40))]
    _, marg = oracle.projection_field((-math.pi, math.pi), RV, POS, R, 0.7, objs,
                                      return_margins=True)
    ex, near = oracle.projection_excuse((-math.pi, math.pi), RV, POS, R, 0.7, objs)
    far = marg >= 1e-9
    assert far.sum() >= 38
    assert not ex[far].any() and not near[far].any()


def test_step_excuse_is_the_union_of_the_pairs():
    """vf_step's per-agent mask equals the OR of projection_excuse's rows of that agent's
    neighbours, and its near count their number."""
    rng = np.random.default_rng(2)
    n, W = 12, 200.0
    st = {"x": rng.uniform(30, 30 + W - 20, n), "y": rng.uniform(30, 30 + W - 20, n),
          "theta": rng.uniform(0, 2 * math.pi, n), "v": np.zeros(n)}
    phis = oracle.linspace(RV)
    # put agent 1 on a midpoint of agent 0's grid
    c0 = (st["x"][0] + R, st["y"][0] + R)
    m = 0.5 * (phis[40] + phis[41]) + st["theta"][0]
    st["x"][1] = c0[0] + 60 * math.cos(m) - R
    st["y"][1] = c0[1] - 60 * math.sin(m) - R
    p = dict(gam=0.1, v0=1.0, alp0=1.0, alp1=0.08, alp2=0.0, bet0=1.0, bet1=0.08, bet2=0.0,
             boundary=0, limit_movement=0, max_vel=3.0, max_th=0.1, width=W, height=W,
             window_pad=30.0, fov0=-math.pi, fov1=math.pi, rv=RV, radius=R, dt=1.0)
    out = oracle.vf_step(st, p, want_excuse=True)
    for i in range(n):
        objs = np.stack([np.delete(st["x"], i), np.delete(st["y"], i)], axis=1)
        ex, near = oracle.projection_excuse((-math.pi, math.pi), RV,
                                            [st["x"][i], st["y"][i]], R, st["theta"][i], objs)
        assert np.array_equal(out["excuse"][i], _raw(ex).max(axis=0)), i
        assert out["near"][i] == near.sum(), i
    assert out["near"][0] >= 1 and out["excuse"][0].any()
