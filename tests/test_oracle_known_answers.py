"""Pin the FP64 oracle (oracle/tcp_oracle.c) against analytic known answers.

The reference has no tests or fixtures; these answers come from closed
forms and literature constants (tests/golden/make_golden.py), never from
the code under test.  CPU only.
"""
import json
import math
import pathlib

import numpy as np
import pytest

GOLD = pathlib.Path(__file__).resolve().parent / "golden"
EPS = 14.399644154020082


def test_pair_closed_forms(orc):
    cases = json.loads((GOLD / "pair_closed_form.json").read_text())
    for c in cases:
        same = c["model"] == "coulomb"
        nel, nion = (2, 0) if same else (1, 1)
        o = orc.Oracle(nel, nion, c["box"], c["box"] / 2, alpha=c["alpha"], rs=c["lam"], lambda_ei=c["lam"],
                       ei="deutsch" if c["model"] == "deutsch" else ("kelbg" if c["model"] == "kelbg" else "coulomb"))
        r = c["r"]
        x = np.array([[r / 2, 0.1, -0.2], [-r / 2, 0.1, -0.2]])
        f, ur = o.force_direct(x)
        assert ur == pytest.approx(c["u"], rel=1e-12, abs=1e-300)
        assert f[0, 0] == pytest.approx(c["f"], rel=1e-12)
        assert f[1, 0] == pytest.approx(-c["f"], rel=1e-12)
        assert abs(f[0, 1]) < 1e-12 * abs(c["f"]) and abs(f[0, 2]) < 1e-12 * abs(c["f"])


def _nacl(nc, a0):
    fcc = np.array([[0, 0, 0], [0, .5, .5], [.5, 0, .5], [.5, .5, 0]])
    cells = np.array([[i, j, k] for i in range(nc) for j in range(nc) for k in range(nc)], dtype=float)
    cat = (cells[:, None, :] + fcc[None]).reshape(-1, 3) * a0
    an = (cells[:, None, :] + fcc[None] + np.array([.5, 0, 0])).reshape(-1, 3) * a0
    return an, cat, a0 / 2


def _cscl(nc, a0):
    cells = np.array([[i, j, k] for i in range(nc) for j in range(nc) for k in range(nc)], dtype=float)
    cat = cells * a0
    an = (cells + 0.5) * a0
    return an, cat, math.sqrt(3.0) * a0 / 2


@pytest.mark.parametrize("lattice,nc", [("NaCl", 4), ("CsCl", 6)])
def test_madelung(orc, lattice, nc):
    mad = json.loads((GOLD / "madelung.json").read_text())[lattice]
    a0 = 5.64
    an, cat, d = (_nacl if lattice == "NaCl" else _cscl)(nc, a0)
    L = nc * a0
    x = np.concatenate([an, cat]) - L / 2 + 0.123
    x = x - L * np.round(x / L)
    rc = L / 2
    alpha = 4.05 / rc
    o = orc.Oracle(len(an), len(cat), L, rc, alpha=alpha, ei="coulomb")
    nmax = int(math.ceil(5.5 * alpha * L / math.pi))
    f, ur, uk = o.force_total(x, recip="ewald", nmax2=nmax * nmax)
    E = (ur + o.Uo) * EPS + uk
    expect = -(len(x) / 2) * mad * EPS / d
    assert E == pytest.approx(expect, rel=2e-7)
    # a perfect lattice is in equilibrium
    assert np.max(np.abs(f)) < 1e-6 * EPS / d ** 2


def _random_system(n, seed, gamma=1.0, lam=0.5):
    from tcp_allpair_gb300.system import make_system
    return make_system(n, gamma=gamma, lam=lam, seed=seed, alpha_rc=3.1)


def test_background_term_makes_a_charged_ewald_sum_alpha_independent(orc):
    """A system with net charge Q: the Ewald total (Ur + Uo) eps + Um does
    not depend on the splitting alpha once Uo carries the neutralising-
    background energy -pi Q^2 / (2 V alpha^2); without it the totals differ
    by pi Q^2 / (2 V) (1/alpha_1^2 - 1/alpha_2^2) eps.  Plain Ewald k-sum and
    real-space sum converged to 1e-9 for both alphas (alpha rc = 4.5, 5)."""
    rng = np.random.default_rng(4)
    nel, nion, L = 40, 24, 20.0
    x = (rng.random((nel + nion, 3)) - 0.5) * L
    rc = L / 2
    Q = -(nel - nion)
    tot, bg = [], []
    for arc in (4.5, 5.0):
        alpha = arc / rc
        o = orc.Oracle(nel, nion, L, rc, alpha=alpha, ei="coulomb", K=0)
        _, ur, uk = o.force_total(x, recip="ewald", nmax2=400)
        tot.append((ur + o.Uo) * EPS + uk)
        bg.append(-math.pi * Q * Q / (2 * L ** 3 * alpha ** 2))
    assert tot[0] == pytest.approx(tot[1], rel=1e-9)
    without = [t - b * EPS for t, b in zip(tot, bg)]
    assert abs(without[0] - without[1]) > 1e3 * abs(tot[0] - tot[1])
    assert abs(without[0] - without[1]) == pytest.approx(abs(bg[0] - bg[1]) * EPS, rel=1e-6)


def test_background_term_vanishes_for_neutral_systems(orc):
    o = orc.Oracle(50, 50, 20.0, 10.0, alpha=0.31, ei="coulomb", K=0)
    assert o.Uo == pytest.approx(-100 * 0.31 / math.sqrt(math.pi), rel=1e-15)


def test_newton3_sum_of_forces(orc):
    s = _random_system(256, 3)
    for ei in ("deutsch", "kelbg"):
        o = orc.Oracle.from_system(s, ei=ei)
        f, _ = o.force_direct(s.x)
        assert np.linalg.norm(f.sum(0)) < 1e-11 * np.abs(f).sum()


def test_rows_match_triangular(orc):
    s = _random_system(300, 4)
    o = orc.Oracle.from_system(s, ei="kelbg")
    f, ur = o.force_direct(s.x)
    fr, ur0 = o.force_direct_rows(s.x, 0, 300)
    assert np.allclose(fr, f, rtol=1e-11, atol=1e-11 * np.abs(f).max())
    assert ur0 == pytest.approx(ur, rel=1e-12)


@pytest.mark.parametrize("order,K,tol", [(4, 32, 3e-4), (5, 32, 5e-5), (6, 48, 2e-6), (8, 64, 2e-7)])
def test_spme_converges_to_ewald(orc, order, K, tol):
    s = _random_system(216, 5)
    s.K, s.order = K, order
    o = orc.Oracle.from_system(s, ei="kelbg")
    fk, uk = o.ewald_ksum(s.x, nmax2=int((5.0 * s.alpha * s.box / math.pi) ** 2))
    fs, us = o.force_spme(s.x)
    assert us == pytest.approx(uk, rel=tol)
    assert orc.rms_rel(fs, fk) < 20 * tol


def test_bspline_moduli_order4_is_reference_formula(orc):
    o = orc.Oracle(2, 0, 10.0, 5.0)
    K = 16
    b = o.bspline_moduli(4, K)
    ref = [36.0 / (4.0 + 2.0 * math.cos(2 * math.pi * m / K)) ** 2 for m in range(K)]   # force.f90:834-839
    assert np.allclose(b, ref, rtol=1e-14)
    # odd orders: finite everywhere (Nyquist index interpolated)
    assert np.all(np.isfinite(o.bspline_moduli(5, K)))


@pytest.mark.parametrize("ei", ["deutsch", "kelbg"])
def test_force_is_minus_gradient(orc, ei):
    s = _random_system(64, 6)
    s.K, s.order = 16, 5
    o = orc.Oracle.from_system(s, ei=ei)

    def energy(x):
        f, ur, um = o.force_total(x, recip="spme")
        return (ur + o.Uo) * EPS + um, f

    E0, f0 = energy(s.x)
    # net-force removal shifts f by sum(f)/N which is ~0 for SPME+direct; undo exactly
    h = 1e-4
    rng = np.random.default_rng(0)
    for i in rng.choice(64, 6, replace=False):
        for k in range(3):
            xp = s.x.copy(); xp[i, k] += h
            xm = s.x.copy(); xm[i, k] -= h
            g = -(energy(xp)[0] - energy(xm)[0]) / (2 * h)
            assert g == pytest.approx(f0[i, k], rel=2e-5, abs=2e-5 * np.abs(f0).max())


def test_charge_scaling_quadratic(orc):
    s = _random_system(128, 7)
    s.K, s.order = 16, 4
    o1 = orc.Oracle.from_system(s, ei="kelbg")
    o2 = orc.Oracle.from_system(s, ei="kelbg", charge_scale=1.3)
    f1, u1, m1 = o1.force_total(s.x)
    f2, u2, m2 = o2.force_total(s.x)
    assert u2 == pytest.approx(1.69 * u1, rel=1e-12)
    assert m2 == pytest.approx(1.69 * m1, rel=1e-12)
    assert o2.Uo == pytest.approx(1.69 * o1.Uo, rel=1e-14)
    assert np.allclose(f2, 1.69 * f1, rtol=1e-10, atol=1e-12)


def test_cutoff_check(orc):
    with pytest.raises(ValueError):
        orc.Oracle(2, 2, 10.0, 5.5)


def test_nve_energy_conservation(orc):
    s = _random_system(128, 8)
    s.K, s.order = 16, 5
    o = orc.Oracle.from_system(s, ei="kelbg")
    x, v = s.x.copy(), s.v.copy()
    f, ur, um = o.force_total(x)
    es = []
    for _ in range(100):
        e = o.md_step(x, v, f, s.dt)
        es.append(e["Epot"] + e["Um"] + 0.5 * (e["mv2el"] + e["mv2ion"]))
    es = np.array(es)
    ke = 0.5 * (e["mv2el"] + e["mv2ion"])
    assert np.max(np.abs(es - es[0])) < 2e-3 * ke


def test_thermostats(orc):
    s = _random_system(128, 9)
    o = orc.Oracle.from_system(s, ei="kelbg", Te=0.5, Ti=0.5)
    for thermo in ("isokin", "berend"):
        v = s.v.copy()
        f = np.zeros_like(v)
        me, mi = o.vverlet2(v, f, s.dt, thermo=thermo)
        if thermo == "isokin":   # vverlet.f90:331-332: exact per-species temperature
            assert me / (3 * s.nel) == pytest.approx(0.5, rel=1e-12)
            assert mi / (3 * s.nion) == pytest.approx(0.5, rel=1e-12)
