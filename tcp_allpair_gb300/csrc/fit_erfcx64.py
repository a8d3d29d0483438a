"""Derive the FP64 tables of the table-driven exp and erfc of the FP64 pair kernels.

erfc(x) = exp(-x^2) erfcx(x) for 0 <= x <= 9: x is rounded to the nearest
multiple of 1/8, x = j/8 + h with |h| <= 1/16 and j = 0..72, and

    erfcx(j/8 + h) = sum_k C[k][j] h^k,   k = 0..DEG,

the least-squares fit in relative error (40-digit mpmath arithmetic) at NPTS
Chebyshev nodes of |h| <= 1/16 (widened by 0.2 %).  Degree 9 leaves an
approximation error of 1.5e-17 relative, below FP64 rounding; evaluated in
FP64 by Horner in h the relative error on [0, 9] is about 3 ulp.  Beyond 9,
erfc(x) < 5e-37 and the kernels take 0.

exp(-z) = 2^(k/64) exp(f), k = rint(-64 z / ln 2), f = -z - k ln2/64,
uses E[i] = 2^(i/64), i = 0..63, rounded to the nearest double.

`python fit_erfcx64.py > erfcx64_table.inc` writes the include file of
pair_math.cuh.
"""
import mpmath as mp

DEG = 9
NSEG = 73          # centres j/8, j = 0..72
STEP = mp.mpf(1) / 8
NPTS = 60


def erfcx(x):
    return mp.erfc(x) * mp.exp(x * x)


def fit_segment(c, hw, deg=DEG, npts=NPTS):
    nodes = [hw * mp.cos(mp.pi * (k + mp.mpf(1) / 2) / npts) for k in range(npts)]
    A = mp.matrix(npts, deg + 1)
    b = mp.matrix(npts, 1)
    for i, h in enumerate(nodes):
        f = erfcx(c + h)
        for j in range(deg + 1):
            A[i, j] = h ** j / f
        b[i] = 1
    co = mp.lu_solve(A.T * A, A.T * b)
    return [co[j] for j in range(deg + 1)]


def tables():
    mp.mp.dps = 40
    hw = STEP / 2 * mp.mpf("1.002")
    segs = [fit_segment(j * STEP, hw) for j in range(NSEG)]
    exp2 = [mp.mpf(2) ** (mp.mpf(i) / 64) for i in range(64)]
    return segs, exp2


def main():
    segs, exp2 = tables()
    out = ["// Generated by fit_erfcx64.py (do not edit): the FP64 erfcx segments",
           f"// C[k][j], erfcx(j/8 + h) = sum_k C[k][j] h^k for |h| <= 1/16, and 2^(i/64).",
           f"constexpr int kErfcxDeg = {DEG}, kErfcxSeg = {NSEG};",
           f"static __constant__ double kErfcxTab[{DEG + 1}][{NSEG}] = {{"]
    for k in range(DEG + 1):
        row = ", ".join(f"{float(segs[j][k]):.17g}" for j in range(NSEG))
        out.append(f"    {{{row}}},")
    out.append("};")
    out.append("static __constant__ double kExp2Tab[64] = {")
    out.append("    " + ", ".join(f"{float(v):.17g}" for v in exp2))
    out.append("};")
    print("\n".join(out))


if __name__ == "__main__":
    main()
