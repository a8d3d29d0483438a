"""Generate the analytic known-answer fixtures in this folder.

The reference ships no tests, fixtures or sample outputs, so the FP64 oracle
is pinned by answers that do not come from any code of this repository:

pair_closed_form.json
    Real-space Ewald pair force and energy of an isolated pair (two
    particles in a box large enough that only the nearest image lies inside
    the cut-off) for the three pair models, evaluated with the closed forms
    below by Python's math module (independent of oracle/ and of the CUDA
    library):
      Coulomb  u = qq erfc(a r)/r,  f = eps qq [erfc(a r) + 2 a r/sqrt(pi) e^{-a^2 r^2}]/r^2
      Deutsch  u = qq (erfc(a r) - e^{-r/rs})/r  (force.f90:135-139)
               f = eps qq [(erfc + 2ar/sqrt(pi) e^{-a^2r^2} - e^{-r/rs})/r^2 - e^{-r/rs}/(r rs)]
      Kelbg    u = qq [erfc(a r)/r - e^{-r^2/l^2}/r + sqrt(pi) erfc(r/l)/l]
               f = -du/dr, from the derivative of each term.
madelung.json
    Madelung constants of the rock-salt (NaCl) and caesium-chloride (CsCl)
    structures referred to the nearest-neighbour distance, from the
    literature (e.g. Kittel, Introduction to Solid State Physics; the
    CRC Handbook): NaCl 1.747564594633182, CsCl 1.762674773070990.

Run from the repository root: python tests/golden/make_golden.py
"""
import json
import math
import pathlib

HERE = pathlib.Path(__file__).resolve().parent
EPS = 14.399644154020082


def pair(model, qq, a, r, lam):
    e1 = math.erfc(a * r)
    g = 2.0 * a * r / math.sqrt(math.pi) * math.exp(-a * a * r * r)
    if model == "coulomb":
        u = qq * e1 / r
        f = EPS * qq * (e1 + g) / r ** 2
    elif model == "deutsch":
        y = math.exp(-r / lam)
        u = qq * (e1 - y) / r
        f = EPS * qq * ((e1 + g - y) / r ** 2 - y / (r * lam))
    else:
        k = math.exp(-r * r / lam ** 2)
        u = qq * (e1 / r - k / r + math.sqrt(math.pi) * math.erfc(r / lam) / lam)
        # -du/dr = qq [e1/r^2 + g/r^2 - k/r^2]
        f = EPS * qq * (e1 + g - k) / r ** 2
    return u, f


def main():
    cases = []
    box = 200.0
    a = 3.1 / (box / 2)
    for model in ("coulomb", "deutsch", "kelbg"):
        for r in (0.3, 1.0, 2.5, 7.0, 20.0, 60.0):
            for lam in (0.5, 3.0):
                qq = -1.0 if model != "coulomb" else 1.0
                u, f = pair(model, qq, a, r, lam)
                cases.append(dict(model=model, box=box, alpha=a, r=r, lam=lam, qq=qq, u=u, f=f))
    (HERE / "pair_closed_form.json").write_text(json.dumps(cases, indent=1))
    (HERE / "madelung.json").write_text(json.dumps({"NaCl": 1.747564594633182, "CsCl": 1.762674773070990},
                                                   indent=1))


if __name__ == "__main__":
    main()
