"""Fits the polynomial of the deterministic 2^y shared by the oracle (or_exp2f) and the
CUDA kernels (gs_exp2f).  Test infrastructure: the coefficients are printed once and
written into both sources; nothing imports this at run time.

Method: y = k + r with k = rint(y), so |r| <= 1/2 and r is exact in FP32; 2^r is written
1 + r c(r) with c of degree 5 (so 1 is exact), and c is fitted to minimise the maximum
relative error of 2^r on Chebyshev nodes by Lawson's iteratively reweighted least squares
(C. L. Lawson, "Contributions to the theory of linear least maximum approximation",
1961), with mpmath references.  The coefficients are rounded to FP32.  Result: relative
error 2.0e-9 before rounding; the FP32 function stays below 0.94 ulp of 2^y over 800k
floats in [-126, 0] (tests/test_oracle.py checks 40k of them and every integer).

The blends take exp(power) as 2^y with y = log2(e) power folded into the conic
(gs_log2_conic): compared with e^x through a Cody & Waite reduction, that drops the
product x log2(e) and the two-part reduction (three operations per pixel and candidate).
"""
import mpmath as mp
import numpy as np


def fit_exp2(deg=6, nodes=4000, iters=60):
    """2^r on |r| <= 1/2 as 1 + r c(r), c of degree deg - 1, fitted for the least maximum
    relative error of 2^r; returns the FP32 coefficients c_1 .. c_deg and the error."""
    mp.mp.dps = 40
    r = np.cos(np.linspace(0.0, np.pi, nodes)) * 0.5
    r = r[np.abs(r) > 1e-12]
    tr = np.array([float(mp.mpf(2) ** mp.mpf(x)) for x in r])
    target = (tr - 1.0) / r
    w = r / tr  # change of 2^r's relative error per unit change of c
    weights = np.ones_like(r)
    V = np.vander(r, deg, increasing=True)
    for _ in range(iters):
        coef, *_ = np.linalg.lstsq(V * (w * weights)[:, None], target * w * weights, rcond=None)
        err = (V @ coef - target) * w
        weights *= (np.abs(err) / np.abs(err).max()) ** 0.3 + 1e-3
    return [np.float32(c) for c in coef], float(np.abs(err).max())


if __name__ == "__main__":
    coef, e = fit_exp2()
    print("max relative error %.3g" % e)
    print("c1..c6:", " ".join(float(c).hex() for c in coef))
