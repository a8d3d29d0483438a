"""The oracle's derivatives (dE/dlambda, Hessian-vector products, dF/dlambda . w,
reverse mode through NOTEMP steps) against central finite differences of the
oracle's own energy, forces and MD steps.  The reference computes no
derivatives, so these pin the derivative oracle that the CUDA library's
adjoint is checked against.  Step h = 1e-4 relative (lambda, charge scale) and
1e-5 a along a unit Gaussian direction (positions; no pair of this
system crosses the cut-off within that step)."""
import numpy as np
import pytest

import oracle
from tcp_allpair_gb300.system import EPS, _wrap, make_system

FD_REL = 1e-6     # central differences at these steps agree to ~1e-8 here


@pytest.fixture(scope="module")
def sys128():
    return make_system(128, gamma=1.0, lam=0.5, seed=3, alpha_rc=3.1, K=16, order=4)


def energy(s, ei, recip, x, **kw):
    o = oracle.Oracle.from_system(s, ei=ei, **kw)
    _, ur, um = o.force_total(x, recip=recip, nmax2=27)
    return (ur + o.Uo) * EPS + (um if recip != "none" else 0.0)


@pytest.mark.parametrize("ei", ["kelbg", "deutsch"])
def test_dE_dlambda_fd(sys128, ei):
    s = sys128
    o = oracle.Oracle.from_system(s, ei=ei)
    lam = s.lambda_ei
    h = 1e-4 * lam
    fd = (energy(s, ei, "spme", s.x, lambda_ei=lam + h, rs=lam + h) -
          energy(s, ei, "spme", s.x, lambda_ei=lam - h, rs=lam - h)) / (2 * h)
    assert o.dE_dlambda(s.x) == pytest.approx(fd, rel=FD_REL)


def test_energy_quadratic_in_charge_scale(sys128):
    s = sys128
    e1 = energy(s, "kelbg", "spme", s.x)
    h = 1e-4
    fd = (energy(s, "kelbg", "spme", s.x, charge_scale=1 + h) - energy(s, "kelbg", "spme", s.x, charge_scale=1 - h)) / (2 * h)
    assert fd == pytest.approx(2 * e1, rel=FD_REL)


@pytest.mark.parametrize("recip", ["spme", "ewald", "none"])
@pytest.mark.parametrize("ei", ["kelbg", "deutsch"])
def test_hvp_fd(sys128, ei, recip):
    s = sys128
    o = oracle.Oracle.from_system(s, ei=ei)
    w = np.random.default_rng(11).normal(size=(s.n, 3))
    hw, dfl = o.hvp(s.x, w, recip=recip, nmax2=27)
    h = 1e-5 * EPS
    fp = o.force_total(_wrap(s.x + h * w, s.box), recip=recip, nmax2=27)[0]
    fm = o.force_total(_wrap(s.x - h * w, s.box), recip=recip, nmax2=27)[0]
    fd = -(fp - fm) / (2 * h)                       # P H w (forces are mean-removed)
    assert oracle.rms_rel(hw - hw.mean(axis=0), fd) < FD_REL
    lam = s.lambda_ei
    hl = 1e-4 * lam
    Fp = oracle.Oracle.from_system(s, ei=ei, lambda_ei=lam + hl, rs=lam + hl).force_total(s.x, recip=recip, nmax2=27)[0]
    Fm = oracle.Oracle.from_system(s, ei=ei, lambda_ei=lam - hl, rs=lam - hl).force_total(s.x, recip=recip, nmax2=27)[0]
    assert dfl == pytest.approx(np.sum((Fp - Fm) / (2 * hl) * w), rel=FD_REL)


def test_hvp_symmetric(sys128):
    """u . (H w) == w . (H u)"""
    s = sys128
    o = oracle.Oracle.from_system(s, ei="kelbg")
    rng = np.random.default_rng(5)
    u, w = rng.normal(size=(s.n, 3)), rng.normal(size=(s.n, 3))
    hw, _ = o.hvp(s.x, w)
    hu, _ = o.hvp(s.x, u)
    assert np.sum(u * hw) == pytest.approx(np.sum(w * hu), rel=1e-12)


@pytest.mark.parametrize("K,M", [(12, 5), (9, 3)])
def test_reverse_md_fd(sys128, K, M):
    s = sys128
    o = oracle.Oracle.from_system(s, ei="kelbg")
    J, dJ = o.reverse_md(s.x, s.v, s.dt, K, M)
    assert J == pytest.approx(o.mean_temperature(s.x, s.v, s.dt, K), rel=1e-14)
    lam = s.lambda_ei
    h = 1e-4 * lam
    Jp = oracle.Oracle.from_system(s, ei="kelbg", lambda_ei=lam + h).mean_temperature(s.x, s.v, s.dt, K)
    Jm = oracle.Oracle.from_system(s, ei="kelbg", lambda_ei=lam - h).mean_temperature(s.x, s.v, s.dt, K)
    assert dJ == pytest.approx((Jp - Jm) / (2 * h), rel=FD_REL)
