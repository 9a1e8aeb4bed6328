"""Helpers shared by the GPU parity tests (seeded swarms, excused-pixel masks)."""
import numpy as np

import oracle


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


def excused_pixels(margins_row, state, i, params, radii=None, band=1e-9):
    """Pixels that a pair within `band` rad of a decision boundary can touch (either
    decision): the union of [t-h-2, t+h+2] (with wrap) of those pairs, via the oracle."""
    rv = int(params["rv"])
    mask = np.zeros(rv, bool)
    js = np.where(margins_row < band)[0]
    for j in js:
        objs = np.array([[state["x"][j], state["y"][j]]])
        sz = None if radii is None else [radii[j]]
        R = params["radius"] if radii is None else radii[i]
        row = oracle.projection_field((params["fov0"], params["fov1"]), rv,
                                      [state["x"][i], state["y"][i]], R, state["theta"][i],
                                      objs, sz, "infinite" if params["boundary"] else "walls",
                                      params["width"], params["height"])[0][::-1]
        on = np.where(row > 0)[0]
        for k in on:
            mask[np.arange(k - 2, k + 3) % rv] = True
        if len(on) == 0:
            mask[:] = True  # a dropped projection could have appeared anywhere near it
    return mask
