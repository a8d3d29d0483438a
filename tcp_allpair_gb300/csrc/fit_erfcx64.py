"""Derive the FP64 tables of the table-driven exp and erfc of the FP64 pair kernels.

The Ewald real-space force needs erfc(x) + 2x/sqrt(pi) exp(-x^2) at x = alpha r,
which is exp(-x^2) Q(x) with

    Q(x) = erfcx(x) + 2x/sqrt(pi),   erfcx(x) = exp(x^2) erfc(x).

For 0 <= x <= 9, x is rounded to the nearest multiple of 1/8, x = j/8 + h with
|h| <= 1/16 and j = 0..72, and

    Q(j/8 + h) = sum_k C[k][j] h^k,   k = 0..DEG,

the least-squares fit in relative error (40-digit mpmath arithmetic) at NPTS
Chebyshev nodes of |h| <= 1/16 (widened by 0.2 %).  Degree 9 leaves an
approximation error below FP64 rounding.  erfc itself, where a kernel needs it
(energies, the Kelbg erfc(r/lambda)), is exp(-x^2) (Q(x) - 2x/sqrt(pi)).
Beyond 9 (erfc(x) < 5e-37, exp(-x^2) < 7e-36) the kernels take 0.

exp(-z) = 2^(k/256) exp(f), k = rint(-256 z / ln 2), f = -z - k ln2/256,
uses E[i] = 2^(i/256), i = 0..255, rounded to the nearest double.

`python fit_erfcx64.py > erfcx64_table.inc` writes the include file of
pair_math.cuh.
"""
import mpmath as mp

DEG = 9
NSEG = 73          # centres j/8, j = 0..72
STEP = mp.mpf(1) / 8
NPTS = 60
NEXP = 256         # exp table entries 2^(i/NEXP)


def erfcx(x):
    return mp.erfc(x) * mp.exp(x * x)


def ewald_q(x):
    return erfcx(x) + 2 * x / mp.sqrt(mp.pi)


def fit_segment(c, hw, deg=DEG, npts=NPTS):
    nodes = [hw * mp.cos(mp.pi * (k + mp.mpf(1) / 2) / npts) for k in range(npts)]
    A = mp.matrix(npts, deg + 1)
    b = mp.matrix(npts, 1)
    for i, h in enumerate(nodes):
        f = ewald_q(c + h)
        for j in range(deg + 1):
            A[i, j] = h ** j / f
        b[i] = 1
    co = mp.lu_solve(A.T * A, A.T * b)
    return [co[j] for j in range(deg + 1)]


def tables():
    mp.mp.dps = 40
    hw = STEP / 2 * mp.mpf("1.002")
    segs = [fit_segment(j * STEP, hw) for j in range(NSEG)]
    exp2 = [mp.mpf(2) ** (mp.mpf(i) / NEXP) for i in range(NEXP)]
    return segs, exp2


def main():
    segs, exp2 = tables()
    out = ["// Generated by fit_erfcx64.py (do not edit): the FP64 segments of",
           "// Q(x) = erfcx(x) + 2x/sqrt(pi), C[k][j] with Q(j/8 + h) = sum_k C[k][j] h^k",
           f"// for |h| <= 1/16, and 2^(i/{NEXP}).",
           f"constexpr int kEwqDeg = {DEG}, kEwqSeg = {NSEG}, kExpTab = {NEXP};",
           f"static __constant__ double kEwqTab[{DEG + 1}][{NSEG}] = {{"]
    for k in range(DEG + 1):
        row = ", ".join(f"{float(segs[j][k]):.17g}" for j in range(NSEG))
        out.append(f"    {{{row}}},")
    out.append("};")
    out.append(f"static __constant__ double kExp2Tab[{NEXP}] = {{")
    out.append("    " + ", ".join(f"{float(v):.17g}" for v in exp2))
    out.append("};")
    print("\n".join(out))


if __name__ == "__main__":
    main()
