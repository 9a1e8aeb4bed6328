"""The FP32 minimal torus image of the group kernels (torus_image2 and the torus window in
abm_gb300/csrc/vpf_step.cu), restated operation by operation in numpy float32 (IEEE
round-to-nearest-even per operation, as the kernel's explicit _rn intrinsics), against exact
rational arithmetic: the minimal image of vf_supcalc.py:70-83 decided on the exact offset and
rounded once to float32.  Adversarial cases put the exact offset on, just inside and just
beyond +-W/2 (differences whose float32 rounding lands exactly on W/2), at the window's edge
(|offset| up to 1.5 W), and at small and large magnitudes.  No GPU: this pins the arithmetic
argument; the GPU tests pin the kernel to the double-float forms bit for bit.
"""
from fractions import Fraction

import numpy as np
import pytest

f32 = np.float32


def _round_f32(fr: Fraction) -> np.float32:
    """fr rounded to the nearest float32, ties to even (no double rounding)."""
    c = f32(float(fr))
    best = None
    for cand in (np.nextafter(c, f32(-np.inf)), c, np.nextafter(c, f32(np.inf))):
        err = abs(Fraction(float(cand)) - fr)
        even = (int(np.array(cand, np.float32).view(np.uint32)) & 1) == 0
        key = (err, not even)
        if best is None or key < best[0]:
            best = (key, cand)
    return best[1]


def _model(v, f, L):
    """torus_image2 for one component: float32 operations in the kernel's order."""
    v, f, L = f32(v), f32(f), f32(L)
    d = f32(v - f)
    nb = f32(v - d)
    t = f32(d + nb)
    e = f32(f32(v - t) + f32(-f + nb))
    h = f32(f32(0.5) * L)
    up = f32(f32(d - h) + e)
    dn = f32(f32(d + h) + e)
    k = f32((f32(1) if up > 0 else f32(0)) + (f32(-1) if dn < 0 else f32(0)))
    # the fused multiply-add d - L k: L k is exact, so one rounding of d - L k
    return f32(f32(d - f32(L * k)) + e), d, e


def _exact(v, f, L):
    s = Fraction(float(f32(v))) - Fraction(float(f32(f)))
    Lf = Fraction(float(f32(L)))
    if s > Lf / 2:
        s -= Lf
    elif s < -Lf / 2:
        s += Lf
    return _round_f32(s)


def _window_ok(v, f, L):
    """The kernel's window test for a one-agent group (bounds rounded inwards)."""
    lo = np.float32(np.nextafter(f32(f32(f) - f32(1.5) * f32(L)), f32(np.inf)))
    hi = np.float32(np.nextafter(f32(f32(f) + f32(1.5) * f32(L)), f32(-np.inf)))
    # the inward rounding of __fadd_ru / __fadd_rd is at least as tight as these bounds when
    # the sum is exact, and these bounds are inside the exact window either way
    return lo <= f32(v) <= hi


def _cases(L, rng, n_random=400):
    L = f32(L)
    h = f32(0.5) * L
    out = []
    for _ in range(n_random):   # anywhere in the window
        f = f32(rng.uniform(-0.5 * L, 1.5 * L))
        v = f32(f + rng.uniform(-1.5 * L, 1.5 * L))
        out.append((v, f))
    for _ in range(n_random):   # offsets within a few ulps of +-W/2
        f = f32(rng.uniform(-0.25 * L, 1.25 * L))
        for sgn in (1, -1):
            v = f32(f + sgn * h)
            for k in range(-3, 4):
                vv = v
                for _ in range(abs(k)):
                    vv = np.nextafter(vv, f32(np.inf) if k > 0 else f32(-np.inf))
                out.append((vv, f))
    # an exact difference h +- tiny whose float32 rounding is exactly h (the e-decided ties)
    for tiny in (1e-5, 3e-6, 1e-7, 2.0 ** -30):
        for base in (f32(0), f32(0.25) * L, L):
            for sgn in (1, -1):
                f = f32(base + sgn * tiny)
                out.append((f32(base + h), f))
                out.append((f32(base - h), f))
    out += [(h, f32(0)), (-h, f32(0)), (f32(0), h), (L, f32(0)), (f32(0), L),
            (f32(1.5) * L, f32(0)), (f32(-1.5) * L, f32(0))]
    return out


@pytest.mark.parametrize("L", [1000.0, 900.0, 5000.0, 777.25, 1024.0, 3.0, 1.0e6])
def test_fp32_minimal_image_is_the_exact_one_rounded_once(L):
    rng = np.random.default_rng(int(L * 4) % 2**31)
    n_wrap = n_ties = 0
    for v, f in _cases(L, rng):
        if not _window_ok(v, f, L):
            continue   # the kernel takes these through the double-float offset
        got, d, e = _model(v, f, L)
        want = _exact(v, f, L)
        assert got == want or (got == 0 and want == 0), (L, float(v), float(f), got, want)
        h = f32(0.5) * f32(L)
        n_wrap += abs(float(d)) > float(h)
        n_ties += (abs(d) == h) and e != 0
    assert n_wrap > 50 and n_ties > 0   # the cases reach the wraps and the e-decided ties


def test_unwrapped_offset_stays_the_rounded_difference():
    """fl(d + e) = d: an offset that does not wrap leaves the model as the plain float32
    difference, the one the walls path uses."""
    rng = np.random.default_rng(5)
    L = f32(1000.0)
    for _ in range(2000):
        f = f32(rng.uniform(0, 1000))
        v = f32(f + rng.uniform(-499, 499))
        got, d, _ = _model(v, f, L)
        assert got == d
