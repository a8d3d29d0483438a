"""Derive the FP64 erfc approximation used by the FP64 Newton-3 pair kernel.

    erfc(x) = exp(-x^2) * t * Q(s),   t = 1 / (1 + P x),
    s = (2 t - (1 + t0)) / (1 - t0) in [-1, 1],   t0 = 1 / (1 + P XMAX),

for 0 <= x <= XMAX.  The kernel already computes exp(-x^2) for the Gaussian
term of the Ewald pair force, so erfc costs one reciprocal and a degree-DEG
polynomial.  Q is the least-squares fit, in relative error and in 40-digit
arithmetic (mpmath), of erfc(x) exp(x^2) / t at NPTS Chebyshev nodes in s.

Evaluated in FP64 (Horner in s, numpy exp for the Gaussian factor) the
relative error on [0, 6] is 4.2e-15, the floor set by the rounding of x^2 in
exp(-x^2) (2 x^2 eps at x = 6); degree 14 gives 2.8e-14.  Run
`python fit_erfc64.py` to print the coefficients in pair_n3_f64.cu (constant
term first).
"""
import mpmath as mp
import numpy as np

P = 0.3
XMAX = 6.0
DEG = 16
NPTS = 400


def fit(p=P, xmax=XMAX, deg=DEG, npts=NPTS):
    mp.mp.dps = 40
    t0 = mp.mpf(1) / (1 + mp.mpf(p) * xmax)
    nodes = [mp.cos(mp.pi * (k + mp.mpf(1) / 2) / npts) for k in range(npts)]

    def f(s):
        t = t0 + (s + 1) / 2 * (1 - t0)
        x = (1 / t - 1) / p
        return mp.erfc(x) * mp.exp(x * x) / t

    A = mp.matrix(npts, deg + 1)
    b = mp.matrix(npts, 1)
    for i, s in enumerate(nodes):
        fv = f(s)
        for j in range(deg + 1):
            A[i, j] = s ** j / fv
        b[i] = 1
    c = mp.lu_solve(A.T * A, A.T * b)
    return [c[j] for j in range(deg + 1)], t0


def fp64_error(c, t0, p=P, xmax=XMAX, n=20001):
    cs = [float(v) for v in c]
    t0 = float(t0)
    worst = 0.0
    for x in np.linspace(0.0, xmax, n):
        t = 1.0 / (1.0 + p * x)
        s = (2.0 * t - (1.0 + t0)) / (1.0 - t0)
        q = cs[-1]
        for cc in cs[-2::-1]:
            q = q * s + cc
        approx = np.exp(-x * x) * t * q
        ref = float(mp.erfc(x))
        worst = max(worst, abs(approx - ref) / ref)
    return worst


if __name__ == "__main__":
    c, t0 = fit()
    print(f"P={P} XMAX={XMAX} DEG={DEG} t0={float(t0):.17g} fp64 max rel error {fp64_error(c, t0):.2e}")
    print(", ".join(f"{float(v):.17g}" for v in c))
