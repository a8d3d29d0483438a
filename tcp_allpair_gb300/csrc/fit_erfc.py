"""Derive the FP32 erfc approximation used by the FP32 pair kernels.

    erfc(x) = exp(-x^2) * t * Q(t),   t = 1 / (1 + P x),   x >= 0

Q is a degree-6 polynomial in t fitted to erfcx(x)/t = erfc(x) exp(x^2)/t by
Lawson's iteratively reweighted least squares, which converges to the minimax
fit in relative error, on x in [0, XMAX].  The arguments the kernels see are
alpha r <= alpha rc (3.1 by default, 3.46 for a 1e-6 Ewald error) and
r/lambda < 6 (the Kelbg terms are skipped beyond 6 lambda).  The exp(-x^2)
factor is shared with the Gaussian term of the Ewald pair force, so a Coulomb
pair costs one ex2 and one reciprocal on the SFU for both erfc and the
Gaussian.

The fit error depends sharply on P: at degree 6, P = 0.36 on [0, 4.5] reaches
a fit error of 1.0e-7 relative, and in FP32 Horner form 4.6e-7 max / 1.2e-7
rms on [0, 4.5] (the FP32 rounding of t dominates), the accuracy the degree-7
fit with P = 0.4 had on [0, 6] (4.4e-7 / 1.15e-7) for one FFMA less per
erfc.  Beyond 4.5 the relative error grows to 6.4e-6 at x = 6, where erfc is
below 2e-10 and the term no longer counts at FP32 precision.  Run
`python fit_erfc.py` to reproduce the coefficients in pair_math.cuh (printed
highest power first).

`python fit_erfc.py --short` fits the degree-5 Q of the Newton-3 kernels'
Ewald term, whose argument alpha r never exceeds alpha rc (3.1 with the
reference's alpha = 3.1/rc, 3.46 for a 1e-6 Ewald error): P = 0.41 on
[0, 3.6] gives 8.5e-7 max / 3.7e-7 rms relative error in FP32 Horner form,
one FMA less per pair (TCP_ERFC5_Q, kErfc5P, kErfc5Xmax).
"""
import sys
import numpy as np
from scipy.special import erfc, erfcx

P = 0.36
DEG = 6
XMAX = 4.5


def fit(p=P, deg=DEG, xmax=XMAX, iters=400):
    t = np.linspace(1.0 / (1.0 + p * xmax), 1.0, 20000)
    x = (1.0 / t - 1.0) / p
    target = erfcx(x) / t
    A = np.vander(t, deg + 1)
    w = np.ones_like(t)
    for _ in range(iters):
        sw = np.sqrt(w) / target
        c, *_ = np.linalg.lstsq(A * sw[:, None], target * sw, rcond=None)
        err = np.abs(A @ c - target) / target
        w = w * (err + 1e-300)
        w /= w.sum()
    return c, float(np.max(np.abs(A @ c - target) / target))


def fp32_error(c, p=P, xmax=6.0):
    x = np.linspace(0.0, xmax, 200001).astype(np.float32)
    t = (np.float32(1.0) / (np.float32(1.0) + np.float32(p) * x)).astype(np.float32)
    q = np.float32(c[0])
    for ci in c[1:]:
        q = (q * t + np.float32(ci)).astype(np.float32)
    approx = np.exp(-x.astype(np.float64) ** 2) * (t * q).astype(np.float64)
    ref = erfc(x.astype(np.float64))
    rel = np.abs(approx - ref) / ref
    return float(rel.max()), float(np.sqrt(np.mean(rel ** 2)))


if __name__ == "__main__":
    p, deg, xmax = (0.41, 5, 3.6) if "--short" in sys.argv else (P, DEG, XMAX)
    c, e = fit(p=p, deg=deg, xmax=xmax)
    mx, rms = fp32_error(c, p=p, xmax=xmax)
    print(f"P={p} DEG={deg} on [0, {xmax}]: fit max rel {e:.3e}; fp32 max rel {mx:.3e}, rms {rms:.3e}")
    print(", ".join(f"{v:.9e}f" for v in c))
