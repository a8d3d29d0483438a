"""Dynamics through the C ABI vs the FP64 oracle: the Langevin (STOCH)
thermostat with its counter-based noise, thermostat periods over the captured
step graph, the plain-Ewald step, and NVE energy conservation."""
import os
import sys

import numpy as np
import pytest

import oracle
import tcp_allpair_gb300 as T

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
pytestmark = pytest.mark.gpu

from philox_ref import stoch_noise  # noqa: E402


def make(n, seed=1, K=16, order=4, alpha_rc=3.1, **kw):
    return T.make_system(n, gamma=1.0, lam=0.5, seed=seed, alpha_rc=alpha_rc, K=K, order=order, **kw)


def test_stoch_thermostat_matches_oracle_noise():
    """VVerletStoch1/Stoch2 (vverlet.f90:9-127) with the GPU's noise stream."""
    s = make(1000, seed=3)
    seed, alpha = 987654321, 0.05
    f0 = np.random.default_rng(0).normal(size=(s.n, 3))
    p = T.params_for(s, precision="fp64", ei="kelbg", recip="spme", thermo="stoch", alpha_lgv=alpha, seed=seed)
    with T.Context(p, s.nel, s.nion) as c:
        c.EWALD_SELF()
        c.upload(x=s.x, v=s.v, f=f0)
        c.VVerlet1(s.dt)
        me, mi = c.VVerlet2(s.dt)            # step counter 0
        gx, gv, gf, _ = c.download()
    o = oracle.Oracle.from_system(s, ei="kelbg", alpha_lgv=alpha)
    x, v, f = s.x.copy(), s.v.copy(), f0.copy()
    o.vverlet1(x, v, f, s.dt, stoch=True)
    eta = stoch_noise(seed, 0, s.n)
    me_o, mi_o = o.vverlet2(v, f, s.dt, thermo="stoch", eta=np.ascontiguousarray(eta))
    assert np.max(np.abs(gx - x)) < 1e-12 * s.box
    assert np.allclose(gv, v, rtol=1e-12, atol=1e-14)
    assert np.allclose(gf, f, rtol=1e-12, atol=1e-12)      # the noise force is added to f (vverlet.f90:95)
    assert me == pytest.approx(me_o, rel=1e-12) and mi == pytest.approx(mi_o, rel=1e-12)


def test_isokin_every_10_steps_in_graph():
    """The N = 16,384 workload's thermostat: isokinetic rescale every 10th step."""
    s = make(1024, seed=4)
    p = T.params_for(s, precision="fp64", ei="kelbg", recip="spme", thermo="isokin", thermo_period=10)
    p.Te = p.Ti = 0.5
    o = oracle.Oracle.from_system(s, ei="kelbg", Te=0.5, Ti=0.5)
    x, v = s.x.copy(), s.v.copy()
    f, _, _ = o.force_total(x)
    with T.Context(p, s.nel, s.nion) as c:
        c.EWALD_SELF()
        c.upload(x=x, v=v, f=f)
        e = c.md_steps(s.dt, 12)
        gx, gv, _, _ = c.download(f=False)
    for k in range(1, 13):
        eo = o.md_step(x, v, f, s.dt, thermo="isokin", apply=(k % 10 == 0))
    assert np.max(np.abs(gx - x)) < 1e-9 * s.box
    assert oracle.rms_rel(gv, v) < 1e-9
    assert e["mv2el"] == pytest.approx(eo["mv2el"], rel=1e-9)


def test_plain_ewald_md_steps():
    """The N = 1024 workload: Kelbg, alpha = 5.6/L, |k| <= 8 (2 pi / L)."""
    s = make(1024, seed=5, alpha_rc=2.8, K=0)
    p = T.params_for(s, precision="fp64", ei="kelbg", recip="ewald", nmax2=64)
    o = oracle.Oracle.from_system(s, ei="kelbg")
    x, v = s.x.copy(), s.v.copy()
    f, _, _ = o.force_total(x, recip="ewald", nmax2=64)
    with T.Context(p, s.nel, s.nion) as c:
        c.EWALD_SELF()
        c.upload(x=x, v=v, f=f)
        e = c.md_steps(s.dt, 5)
        gx, gv, _, _ = c.download(f=False)
    for _ in range(5):
        eo = o.md_step(x, v, f, s.dt, recip="ewald", nmax2=64)
    assert np.max(np.abs(gx - x)) < 1e-9 * s.box
    assert e["Um"] == pytest.approx(eo["Um"], rel=1e-9)
    assert e["Epot"] == pytest.approx(eo["Epot"], rel=1e-9)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_nve_energy_drift(precision):
    """Total energy Epot + Um + (mv2el + mv2ion)/2 (result.f90:312-320) over 300
    NVE steps at N = 4096 (SPME 32^3, order 5)."""
    s = make(4096, seed=6, K=32, order=5)
    p = T.params_for(s, precision=precision, ei="kelbg", recip="spme")
    with T.Context(p, s.nel, s.nion) as c:
        c.EWALD_SELF()
        c.upload(x=s.x, v=s.v)
        c.force()
        es = []
        for _ in range(6):
            e = c.md_steps(s.dt, 50)
            es.append(e["Epot"] + e["Um"] + 0.5 * (e["mv2el"] + e["mv2ion"]))
        ke = 0.5 * (e["mv2el"] + e["mv2ion"])
    es = np.array(es)
    assert np.all(np.isfinite(es))
    assert np.max(np.abs(es - es[0])) < 5e-3 * ke


def test_nve_drift_fp32c_tracks_fp64():
    """500 NVE steps at N = 4096 (the headline run length): the total-energy
    drift of the compensated-FP32 step stays at the level of the FP64 step's
    (the drift is the integrator's, not the pair arithmetic's)."""
    s = make(4096, seed=7, K=32, order=5)
    drift = {}
    for prec in ("fp64", "fp32c"):
        p = T.params_for(s, precision=prec, ei="kelbg", recip="spme")
        with T.Context(p, s.nel, s.nion) as c:
            c.EWALD_SELF()
            c.upload(x=s.x, v=s.v)
            c.force()
            e = c.md_steps(s.dt, 1)
            E0 = e["Epot"] + e["Um"] + 0.5 * (e["mv2el"] + e["mv2ion"])
            worst = 0.0
            for _ in range(10):
                e = c.md_steps(s.dt, 50)
                E = e["Epot"] + e["Um"] + 0.5 * (e["mv2el"] + e["mv2ion"])
                worst = max(worst, abs(E - E0) / abs(E0))
        drift[prec] = worst
    assert drift["fp64"] < 1e-3
    assert drift["fp32c"] < 2.0 * drift["fp64"] + 1e-6, drift
