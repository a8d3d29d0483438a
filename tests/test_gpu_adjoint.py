"""Derivatives through the C ABI (tcp_adjoint_energy, tcp_hvp, tcp_reverse_md)
on the differentiation workload (N = 4096, Gamma = 1, lambda = 0.5 a, Kelbg,
SPME 32^3 order 4) against central finite differences of the library's own
FP64 energies / forces / MD steps (h = 1e-4 relative for lambda and the charge
scale, 1e-6 a along a unit Gaussian direction for positions) and against the
FP64 oracle (the reference gradient).  The position step is small because the
real-space sum is truncated at rc: the force jumps when a pair crosses rc, and
at h = 1e-5 a about 40 of the 8.4e6 pairs of this system cross it (central
differences then differ from H w by 7e-5 RMS, for the oracle as well).

Tolerances: FP64 adjoint vs central differences 1e-5 relative (the target);
FP64 library vs FP64 oracle 1e-9; compensated-FP32 derivatives vs the FP64
reference gradient: energy derivatives and HVP 1e-5, reverse mode 1e-3 (the
FP32 trajectory itself departs from the FP64 one over 200 steps)."""
import numpy as np
import pytest

import oracle
import tcp_allpair_gb300 as T
from tcp_allpair_gb300.system import EPS, _wrap, make_config_system

pytestmark = pytest.mark.gpu

GRAD_REL = 1e-5


def ctx_for(s, **kw):
    c = T.Context(T.params_for(s, **kw), s.nel, s.nion)
    c.EWALD_SELF()
    c.upload(x=s.x, v=s.v)
    return c


def with_params(p, **kw):
    q = type(p).from_buffer_copy(p)
    for k, v in kw.items():
        setattr(q, k, v)
    return q


def potential(c):
    e = c.force()
    return e["Epot"] + e["Um"]


@pytest.fixture(scope="module")
def sys4096():
    return make_config_system("n4096_adjoint", seed=0)


@pytest.fixture(scope="module")
def w4096(sys4096):
    return np.random.default_rng(2024).normal(size=(sys4096.n, 3))


@pytest.fixture(scope="module")
def oracle_ref(sys4096, w4096):
    s = sys4096
    o = oracle.Oracle.from_system(s, ei="kelbg")
    _, ur, um = o.force_total(s.x)
    hw, dfl = o.hvp(s.x, w4096)
    return dict(E=(ur + o.Uo) * EPS + um, dEdl=o.dE_dlambda(s.x), hw=hw, dfl=dfl)


def test_energy_gradients_fp64(sys4096, oracle_ref):
    s = sys4096
    with ctx_for(s, precision="fp64", ei="kelbg", recip="spme") as c:
        E, dl, ds = c.adjoint_energy()
        p = c.params
        lam, h = s.lambda_ei, 1e-4
        c.set_params(with_params(p, lambda_ei=lam * (1 + h), rs=lam * (1 + h)))
        ep = potential(c)
        c.set_params(with_params(p, lambda_ei=lam * (1 - h), rs=lam * (1 - h)))
        em = potential(c)
        fd_l = (ep - em) / (2 * h * lam)
        c.set_params(with_params(p, charge_scale=1 + h))
        ep = potential(c)
        c.set_params(with_params(p, charge_scale=1 - h))
        em = potential(c)
        fd_s = (ep - em) / (2 * h)
    assert abs(dl - fd_l) <= GRAD_REL * abs(fd_l), (dl, fd_l)
    assert abs(ds - fd_s) <= GRAD_REL * abs(fd_s), (ds, fd_s)
    assert E == pytest.approx(oracle_ref["E"], rel=1e-10)
    assert dl == pytest.approx(oracle_ref["dEdl"], rel=1e-10)


def test_energy_gradients_fp32c(sys4096, oracle_ref):
    s = sys4096
    with ctx_for(s, precision="fp32c", ei="kelbg", recip="spme") as c:
        E, dl, ds = c.adjoint_energy()
        _, _, f, _ = c.download(x=False, v=False, f=True)
    assert dl == pytest.approx(oracle_ref["dEdl"], rel=GRAD_REL)
    assert ds == pytest.approx(2 * oracle_ref["E"], rel=GRAD_REL)
    assert np.all(f == 0.0)          # stored forces kept (none were computed)


def test_hvp_fp64(sys4096, w4096, oracle_ref):
    s, w = sys4096, w4096
    with ctx_for(s, precision="fp64", ei="kelbg", recip="spme") as c:
        hw, dfl = c.hvp(w)
        h = 1e-6 * EPS
        c.upload(x=_wrap(s.x + h * w, s.box))
        c.force()
        fp = c.download(x=False, v=False, f=True)[2]
        c.upload(x=_wrap(s.x - h * w, s.box))
        c.force()
        fm = c.download(x=False, v=False, f=True)[2]
        p = c.params
        lam, hl = s.lambda_ei, 1e-4 * s.lambda_ei
        c.upload(x=s.x)
        c.set_params(with_params(p, lambda_ei=lam + hl))
        c.force()
        Fp = c.download(x=False, v=False, f=True)[2]
        c.set_params(with_params(p, lambda_ei=lam - hl))
        c.force()
        Fm = c.download(x=False, v=False, f=True)[2]
    fd = -(fp - fm) / (2 * h)
    assert oracle.rms_rel(hw - hw.mean(axis=0), fd) < GRAD_REL
    assert dfl == pytest.approx(np.sum((Fp - Fm) / (2 * hl) * w), rel=GRAD_REL)
    assert oracle.rms_rel(hw, oracle_ref["hw"]) < 1e-9
    assert dfl == pytest.approx(oracle_ref["dfl"], rel=1e-9)


def test_hvp_fp32c(sys4096, w4096, oracle_ref):
    with ctx_for(sys4096, precision="fp32c", ei="kelbg", recip="spme") as c:
        hw, dfl = c.hvp(w4096)
    assert oracle.rms_rel(hw, oracle_ref["hw"]) < GRAD_REL
    assert dfl == pytest.approx(oracle_ref["dfl"], rel=GRAD_REL)


@pytest.mark.parametrize("ei,recip", [("deutsch", "ewald"), ("kelbg", "none"), ("coulomb", "spme")])
def test_hvp_models_vs_oracle(ei, recip):
    s = T.make_system(1000, gamma=1.0, lam=0.5, seed=9, alpha_rc=3.1, K=16, order=5)
    w = np.random.default_rng(3).normal(size=(s.n, 3))
    o = oracle.Oracle.from_system(s, ei=ei)
    hw_o, dfl_o = o.hvp(s.x, w, recip=recip, nmax2=27)
    with ctx_for(s, precision="fp64", ei=ei, recip=recip, nmax2=27) as c:
        hw, dfl = c.hvp(w)
        _, dl, _ = c.adjoint_energy()
    assert oracle.rms_rel(hw, hw_o) < 1e-9
    if ei == "coulomb":
        assert dfl == 0.0 and dl == 0.0
    else:
        assert dfl == pytest.approx(dfl_o, rel=1e-9)
        assert dl == pytest.approx(o.dE_dlambda(s.x), rel=1e-10)


@pytest.mark.parametrize("ei,recip", [("kelbg", "spme"), ("deutsch", "ewald"), ("kelbg", "none")])
def test_reverse_md_vs_oracle(ei, recip):
    """Small case (5 checkpointed segments, the last one partial) against the
    oracle's reverse mode, and the state after the sweep against plain steps."""
    s = T.make_system(256, gamma=1.0, lam=0.5, seed=21, alpha_rc=3.1, K=16, order=4)
    o = oracle.Oracle.from_system(s, ei=ei)
    Jo, dJo = o.reverse_md(s.x, s.v, s.dt, 18, 4, recip=recip, nmax2=27)
    with ctx_for(s, precision="fp64", ei=ei, recip=recip, nmax2=27) as c:
        J, dJ = c.reverse_md(s.dt, 18, 4)
        x, v, _, _ = c.download(x=True, v=True, f=False)
    assert J == pytest.approx(Jo, rel=1e-11)
    assert dJ == pytest.approx(dJo, rel=1e-8)
    xo, vo = s.x.copy(), s.v.copy()
    f, _, _ = o.force_total(xo, recip=recip, nmax2=27)
    for _ in range(18):
        o.md_step(xo, vo, f, s.dt, recip=recip, nmax2=27)
    assert np.max(np.abs(x - xo)) < 1e-9 * s.box
    assert oracle.rms_rel(v, vo) < 1e-9


def test_reverse_md_fp32c_small_vs_oracle():
    s = T.make_system(512, gamma=1.0, lam=0.5, seed=22, alpha_rc=3.1, K=16, order=4)
    o = oracle.Oracle.from_system(s, ei="kelbg")
    Jo, dJo = o.reverse_md(s.x, s.v, s.dt, 20, 5)
    with ctx_for(s, precision="fp32c", ei="kelbg", recip="spme") as c:
        J, dJ = c.reverse_md(s.dt, 20, 5)
    assert J == pytest.approx(Jo, rel=1e-6)
    assert dJ == pytest.approx(dJo, rel=1e-4)


def mean_temperature(c, s, dt, K):
    c.upload(x=s.x, v=s.v)
    c.force()
    acc = 0.0
    for _ in range(K):
        e = c.md_steps(dt, 1)
        acc += e["mv2el"] + e["mv2ion"]
    return acc / (3.0 * s.n * K)


@pytest.fixture(scope="module")
def reverse_fp64(sys4096):
    s = sys4096
    with ctx_for(s, precision="fp64", ei="kelbg", recip="spme") as c:
        J, dJ = c.reverse_md(s.dt, 200, 20)
        p = c.params
        lam, h = s.lambda_ei, 1e-4
        J0 = mean_temperature(c, s, s.dt, 200)
        c.set_params(with_params(p, lambda_ei=lam * (1 + h)))
        Jp = mean_temperature(c, s, s.dt, 200)
        c.set_params(with_params(p, lambda_ei=lam * (1 - h)))
        Jm = mean_temperature(c, s, s.dt, 200)
    return dict(J=J, dJ=dJ, J0=J0, fd=(Jp - Jm) / (2 * h * lam))


def test_reverse_md_fp64_vs_fd(reverse_fp64):
    r = reverse_fp64
    assert r["J"] == pytest.approx(r["J0"], rel=1e-10)
    assert abs(r["dJ"] - r["fd"]) <= GRAD_REL * abs(r["fd"]), r


def test_reverse_md_fp32c_vs_fp64(sys4096, reverse_fp64):
    s = sys4096
    with ctx_for(s, precision="fp32c", ei="kelbg", recip="spme") as c:
        J, dJ = c.reverse_md(s.dt, 200, 20)
    assert J == pytest.approx(reverse_fp64["J"], rel=1e-5)
    assert dJ == pytest.approx(reverse_fp64["dJ"], rel=1e-3), (dJ, reverse_fp64["dJ"])


def test_reverse_md_rejects_thermostat():
    s = T.make_system(256, seed=1, alpha_rc=3.1, K=16)
    with ctx_for(s, precision="fp64", thermo="isokin") as c:
        with pytest.raises(T.TcpError):
            c.reverse_md(s.dt, 4, 2)


@pytest.mark.parametrize("r_over_lam", [1e-2, 0.1, 0.3, 1.0])
def test_hvp_fp32c_close_kelbg_pair(r_over_lam):
    """One electron and one ion at r = (0.01 .. 1) lambda: the FP32C
    Hessian-vector product and dF/dlambda.w against the oracle (close pairs
    take the FP64 radial functions; their FP32 form cancels to r^2/lambda^2)."""
    s = T.make_system(2, gamma=1.0, lam=0.5, seed=1, alpha_rc=3.1, K=8, order=4)
    u = np.array([0.48, -0.6, 0.64])
    x = np.zeros((2, 3))
    x[1] = r_over_lam * s.lambda_ei * u / np.linalg.norm(u)
    w = np.array([[0.3, -0.2, 0.9], [-0.5, 0.4, 0.1]])
    hw_o, dfl_o = oracle.Oracle.from_system(s, ei="kelbg").hvp(x, w, recip="none")
    with T.Context(T.params_for(s, precision="fp32c", ei="kelbg", recip="none"), 1, 1) as c:
        c.EWALD_SELF()
        c.upload(x=x, v=np.zeros((2, 3)))
        hw, dfl = c.hvp(w)
    assert oracle.rms_rel(hw, hw_o) < 2e-5
    assert dfl == pytest.approx(dfl_o, rel=2e-5)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
@pytest.mark.parametrize("ei", ["kelbg", "deutsch", "coulomb"])
def test_newton3_adjoint_matches_ordered(precision, ei):
    """The Newton-3 real-space H w / dE/dlambda / dF/dlambda.w (default)
    against the ordered-pair sums (TCP_FLAG_DETERMINISTIC) on 700 electrons
    and 300 ions (ragged tiles, unequal species)."""
    s = T.make_system(1000, gamma=1.0, lam=0.5, seed=12, alpha_rc=3.1, K=16, order=4)
    s.nel, s.nion = 700, 300
    w = np.random.default_rng(5).normal(size=(s.n, 3))
    out = {}
    for det in (False, True):
        with ctx_for(s, precision=precision, ei=ei, recip="none") as c:
            if det:
                c.set_flags(T.FLAG_ENERGY | T.FLAG_DETERMINISTIC)
            hw, dfl = c.hvp(w)
            _, dl, _ = c.adjoint_energy()
        out[det] = (hw, dfl, dl)
    tol = 1e-12 if precision == "fp64" else 2e-6
    assert oracle.rms_rel(out[False][0], out[True][0]) < tol
    if ei == "coulomb":
        assert out[False][1] == 0.0 and out[False][2] == 0.0
    else:
        assert out[False][1] == pytest.approx(out[True][1], rel=tol)
        assert out[False][2] == pytest.approx(out[True][2], rel=tol)
