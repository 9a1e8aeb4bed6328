"""Fit the FP32 arctangent polynomial used by the pair kernels (vpf_common.cuh).

atan(r) on r in [0, 1] is approximated as r * P(r^2), P of degree DEG, by a near-minimax
fit of the ABSOLUTE error: Lawson's iteratively reweighted least squares on a dense grid
(C. L. Lawson, "Contributions to the theory of linear least maximum approximation", 1961),
in float64, then the coefficients are rounded to float32.  The script prints the
coefficients in the C initialiser form used by the header and the maximum absolute error of
the rounded polynomial evaluated in float64 (the GPU's float32 Horner evaluation adds a few
ulps on top; the kernels' decision bands are sized for 1e-6 rad total and the GPU tests
check the measured error).

    python abm_gb300/csrc/fit_atan.py
"""
import numpy as np

DEG = 8


def fit(deg=DEG, n=20000, iters=400):
    r = np.cos(np.linspace(np.pi, 0, n)) * 0.5 + 0.5          # Chebyshev-clustered in [0,1]
    s = r * r
    A = r[:, None] * s[:, None] ** np.arange(deg + 1)[None, :]
    y = np.arctan(r)
    w = np.ones(n) / n
    c = None
    for _ in range(iters):
        sw = np.sqrt(w)
        c, *_ = np.linalg.lstsq(A * sw[:, None], y * sw, rcond=None)
        err = np.abs(A @ c - y)
        w = w * err
        w /= w.sum()
    return c


def main():
    c = fit()
    c32 = c.astype(np.float32)
    r = np.linspace(0, 1, 2_000_001)
    s = r * r
    p = np.zeros_like(r)
    for k in range(DEG, -1, -1):
        p = p * s + float(c32[k])
    err = np.max(np.abs(r * p - np.arctan(r)))
    print("coefficients (c0 .. c%d):" % DEG)
    print(", ".join("%.9ef" % float(v) for v in c32))
    print("max |r*P(r^2) - atan(r)| on [0,1] with float32 coefficients: %.3e" % err)


if __name__ == "__main__":
    main()
