"""CUDA library (through the C ABI) vs the FP64 oracle on identical seeded inputs.

Tolerances: the FP64 kernels agree with the oracle to summation-order
rounding (1e-11 relative); the compensated-FP32 pair kernel meets the
RMS relative force error bound 2e-6 of the FP32 path.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
import tcp_allpair_gb300 as T
from tcp_allpair_gb300 import _abi

pytestmark = pytest.mark.gpu

FP32_FORCE_RMS = 2e-6       # RMS relative force error bound of the FP32C path
FP64_REL = 1e-11


def make(n, seed=1, K=16, order=4, lam=0.5, gamma=1.0, alpha_rc=3.1, **kw):
    return T.make_system(n, gamma=gamma, lam=lam, seed=seed, alpha_rc=alpha_rc, K=K, order=order, **kw)


def ctx_for(s, **kw):
    p = T.params_for(s, **kw)
    c = T.Context(p, s.nel, s.nion)
    c.EWALD_SELF()
    c.upload(x=s.x, v=s.v)
    return c


@pytest.mark.parametrize("ei", ["deutsch", "kelbg", "coulomb"])
@pytest.mark.parametrize("n", [1024, 1000])
def test_direct_fp64(ei, n):
    s = make(n, seed=2)
    o = oracle.Oracle.from_system(s, ei=ei)
    fo, uo = o.force_direct(s.x)
    with ctx_for(s, precision="fp64", ei=ei, recip="none") as c:
        ur = c.Force_direct_self()
        _, _, f, _ = c.download(x=False, v=False, f=True)
    assert ur == pytest.approx(uo, rel=FP64_REL)
    assert oracle.rms_rel(f, fo) < FP64_REL


@pytest.mark.parametrize("deterministic", [False, True])
@pytest.mark.parametrize("ei", ["deutsch", "kelbg"])
def test_direct_fp64_at_rounding_level(ei, deterministic):
    """The FP64 kernels' table-driven exp / erfc and Newton rsqrt (about
    2e-16 relative each) keep the direct sum at FP64 rounding level: RMS force
    and energy within 1e-13 of the oracle (math-library erfc / exp / sqrt),
    a hundred times tighter than the general FP64 bound."""
    s = make(2048, seed=31, lam=0.3)
    o = oracle.Oracle.from_system(s, ei=ei)
    fo, uo = o.force_direct(s.x)
    with ctx_for(s, precision="fp64", ei=ei, recip="none") as c:
        if deterministic:
            c.set_flags(T.FLAG_ENERGY | T.FLAG_DETERMINISTIC)
        ur = c.Force_direct_self()
        _, _, f, _ = c.download(x=False, v=False, f=True)
    err = oracle.rms_rel(f, fo)
    assert err < 1e-13, err
    assert ur == pytest.approx(uo, rel=1e-13)


@pytest.mark.parametrize("ei", ["deutsch", "kelbg", "coulomb"])
@pytest.mark.parametrize("n", [1024, 4096, 777])
def test_direct_fp32c(ei, n):
    s = make(n, seed=3)
    o = oracle.Oracle.from_system(s, ei=ei)
    fo, uo = o.force_direct(s.x)
    with ctx_for(s, precision="fp32c", ei=ei, recip="none") as c:
        ur = c.Force_direct_self()
        _, _, f, _ = c.download(x=False, v=False, f=True)
    err = oracle.rms_rel(f, fo)
    assert err < FP32_FORCE_RMS, err
    assert ur == pytest.approx(uo, rel=2e-5)


@pytest.mark.parametrize("order,K", [(4, 16), (5, 32), (6, 24), (4, 30), (5, 96), (4, 128)])
def test_spme_vs_oracle(order, K):
    """FP64 SPME against the oracle; the meshes take the spread's three row
    groupings (2 rows per warp below 8,192 (y, z) columns, 4 below 16,384,
    8 above)."""
    s = make(2000, seed=4, K=K, order=order)
    o = oracle.Oracle.from_system(s, ei="kelbg")
    fo, umo = o.force_spme(s.x)
    with ctx_for(s, precision="fp64", ei="kelbg", recip="spme") as c:
        um = c.Force_SPME4()
        _, _, _, fr = c.download(x=False, v=False, f=False, frec=True)
    assert um == pytest.approx(umo, rel=1e-11)
    assert oracle.rms_rel(fr, fo) < 1e-10


@pytest.mark.parametrize("order,K,tol", [(4, 16, 6e-6), (5, 32, 1e-6), (6, 24, 1e-6)])
def test_spme_fp32_mode_vs_oracle(order, K, tol):
    """FP32C mode: compensated-FP32 charge accumulation, FP32 transforms and
    gather.  The reciprocal forces come from spline-derivative sums over a
    smooth potential, which amplify the FP32 rounding of the transforms: the
    measured RMS errors of these three cases on GB300 were 2.9e-6, 4.6e-7 and
    3.2e-7; the bounds are about twice that (TCP_PREC_FP32C_R64 runs the
    chain in FP64)."""
    s = make(2000, seed=4, K=K, order=order)
    o = oracle.Oracle.from_system(s, ei="kelbg")
    fo, umo = o.force_spme(s.x)
    with ctx_for(s, precision="fp32c", ei="kelbg", recip="spme") as c:
        um = c.Force_SPME4()
        _, _, _, fr = c.download(x=False, v=False, f=False, frec=True)
    assert um == pytest.approx(umo, rel=1e-6)
    assert oracle.rms_rel(fr, fo) < tol


def test_ewald_ksum_vs_oracle():
    s = make(1024, seed=5, alpha_rc=2.8)   # alpha = 5.6/L
    o = oracle.Oracle.from_system(s, ei="kelbg")
    fo, uko = o.ewald_ksum(s.x, 64)
    with ctx_for(s, precision="fp64", ei="kelbg", recip="ewald", nmax2=64) as c:
        uk = c.Force_SPME4()
        _, _, _, fr = c.download(x=False, v=False, f=False, frec=True)
    assert uk == pytest.approx(uko, rel=1e-11)
    assert oracle.rms_rel(fr, fo) < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_total_force_and_energies(precision):
    s = make(2048, seed=6, K=32, order=5)
    o = oracle.Oracle.from_system(s, ei="kelbg")
    fo, uro, umo = o.force_total(s.x, recip="spme")
    with ctx_for(s, precision=precision, ei="kelbg", recip="spme") as c:
        e = c.force()
        _, _, f, _ = c.download(x=False, v=False, f=True)
    tol = FP64_REL if precision == "fp64" else FP32_FORCE_RMS
    assert oracle.rms_rel(f, fo) < tol
    assert e["Um"] == pytest.approx(umo, rel=1e-11 if precision == "fp64" else 1e-6)
    assert e["Ur"] == pytest.approx(uro, rel=1e-11 if precision == "fp64" else 2e-5)
    assert e["Uo"] == pytest.approx(o.Uo, rel=1e-14)
    assert e["Epot"] == pytest.approx((e["Ur"] + e["Uo"]) * T.EPS, rel=1e-14)
    assert np.linalg.norm(f.sum(0)) < 1e-9 * np.abs(f).sum()       # REMOVE_RIGIDMTN applied


def test_granular_routines_compose_like_force():
    s = make(1536, seed=7, K=16, order=4)
    with ctx_for(s, precision="fp64", ei="deutsch", recip="spme") as c:
        um = c.Force_SPME4()
        ur = c.Force_direct_self()
        c.SPME_SUM()
        c.REMOVE_RIGIDMTN()
        _, _, f1, _ = c.download(x=False, v=False, f=True)
        e = c.force()
        _, _, f2, _ = c.download(x=False, v=False, f=True)
    assert np.allclose(f1, f2, rtol=1e-13, atol=1e-13 * np.abs(f2).max())
    assert e["Ur"] == pytest.approx(ur, rel=1e-13) and e["Um"] == pytest.approx(um, rel=1e-13)


@pytest.mark.parametrize("thermo", ["notemp", "isokin", "berend"])
def test_verlet_halves_vs_oracle(thermo):
    s = make(1000, seed=8, K=16)
    rng = np.random.default_rng(0)
    f0 = rng.normal(size=(s.n, 3))
    o = oracle.Oracle.from_system(s, ei="kelbg", Te=0.7, Ti=0.3, tau=2.0)
    p = T.params_for(s, precision="fp64", ei="kelbg", recip="spme", thermo=thermo, tau=2.0)
    p.Te, p.Ti = 0.7, 0.3
    x, v = s.x.copy(), s.v.copy()
    with T.Context(p, s.nel, s.nion) as c:
        c.EWALD_SELF()
        c.upload(x=x, v=v, f=f0)
        c.VVerlet1(s.dt)
        me, mi = c.VVerlet2(s.dt)
        gx, gv, _, _ = c.download(x=True, v=True, f=False)
    f = f0.copy()
    o.vverlet1(x, v, f, s.dt)
    me_o, mi_o = o.vverlet2(v, f, s.dt, thermo=thermo)
    assert np.allclose(gx, x, rtol=0, atol=1e-12 * s.box)
    assert np.allclose(gv, v, rtol=1e-13, atol=1e-15)
    assert me == pytest.approx(me_o, rel=1e-12) and mi == pytest.approx(mi_o, rel=1e-12)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32c", 1e-5)])
def test_md_steps_graph_vs_oracle(precision, tol):
    s = make(1024, seed=9, K=16, order=4)
    o = oracle.Oracle.from_system(s, ei="kelbg")
    x, v = s.x.copy(), s.v.copy()
    f, _, _ = o.force_total(x)
    with ctx_for(s, precision=precision, ei="kelbg", recip="spme") as c:
        c.upload(f=f)
        e = c.md_steps(s.dt, 5)
        gx, gv, gf, _ = c.download()
    for _ in range(5):
        eo = o.md_step(x, v, f, s.dt)
    assert np.max(np.abs(gx - x)) < tol * s.box
    assert oracle.rms_rel(gv, v) < tol
    assert e["Epot"] == pytest.approx(eo["Epot"], rel=10 * tol)
    assert e["mv2el"] == pytest.approx(eo["mv2el"], rel=tol)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-9), ("fp32c", 2e-5)])
def test_md_trajectory_200_steps_vs_oracle(precision, tol):
    """200 graph-launched steps against the oracle stepped alongside from the
    same start: positions, velocities and Epot after every 50."""
    s = make(1024, seed=12, K=16, order=4)
    o = oracle.Oracle.from_system(s, ei="kelbg")
    x, v = s.x.copy(), s.v.copy()
    f, _, _ = o.force_total(x)
    with ctx_for(s, precision=precision, ei="kelbg", recip="spme") as c:
        c.upload(f=f)
        for block in range(4):
            e = c.md_steps(s.dt, 50)
            gx, gv, _, _ = c.download()
            for _ in range(50):
                eo = o.md_step(x, v, f, s.dt)
            assert np.max(np.abs(gx - x)) < tol * s.box, block
            assert oracle.rms_rel(gv, v) < tol, block
            assert e["Epot"] == pytest.approx(eo["Epot"], rel=10 * tol), block


def test_finit_vs_oracle():
    s = make(1024, seed=10, K=16)
    o = oracle.Oracle.from_system(s, ei="deutsch")
    x = s.x.copy()
    fo, uro, umo = o.finit(x, s.v, s.dt)
    with ctx_for(s, precision="fp64", ei="deutsch", recip="spme") as c:
        e = c.Finit(s.dt)
        gx, _, gf, _ = c.download(v=False)
    assert oracle.rms_rel(gf, fo) < FP64_REL
    assert np.max(np.abs(gx - x)) < 1e-12 * s.box
    assert e["Ur"] == pytest.approx(uro, rel=FP64_REL)


def test_rdf_vdf_histograms():
    s = make(1024, seed=12, K=16)
    o = oracle.Oracle.from_system(s, ei="deutsch")
    _, _, h = o.force_direct(s.x, rdf=True)
    with ctx_for(s, precision="fp64", ei="deutsch", recip="none") as c:
        c.set_flags(T.FLAG_ENERGY | T.FLAG_RDF | T.FLAG_VDF)
        c.Force_direct_self()
        _, _, gf, _ = c.download(x=False, v=False, f=True)
        c.VVerlet2(s.dt)
        rdf, vdf = c.histograms(reset=True)
        rdf2, vdf2 = c.histograms()
    assert np.array_equal(rdf, h)                 # +2 per pair inside rc, force.f90:99-103
    assert rdf2.sum() == 0 and vdf2.sum() == 0    # reset as DUMP does, result.f90:264-268
    v, f = s.v.copy(), gf.copy()
    _, _, hv = o.vverlet2(v, f, s.dt, vdf=True)
    assert np.array_equal(vdf, hv)                # vverlet.f90:201-204


def test_pt_roundtrip_and_stride():
    s = make(300, seed=13, K=16)
    qel, qion = s.to_pt()
    qel["ff"] = np.random.default_rng(1).normal(size=(s.nel, 3))
    qion["ff"] = np.random.default_rng(2).normal(size=(s.nion, 3))
    p = T.params_for(s, precision="fp64", recip="spme")
    with T.Context(p, s.nel, s.nion) as c:
        c.upload_pt(qel, qion)
        a = np.zeros_like(qel)
        b = np.zeros_like(qion)
        a["id"], b["id"] = 7, 9
        c.download_pt(a, b)
    for k in ("xx", "xv", "ff"):
        assert np.array_equal(a[k], qel[k]) and np.array_equal(b[k], qion[k])
    assert np.all(a["id"] == 7) and np.all(b["id"] == 9)     # other fields untouched


@pytest.mark.parametrize("direct", ["1", "0"])
def test_transfer_paths(direct, monkeypatch):
    """PT records and (N, 3) arrays through both transfer paths: the device
    reading / writing the caller's host arrays in place (where the device can
    address pageable memory) and the staged copies (TCP_HOST_DIRECT=0)."""
    monkeypatch.setenv("TCP_HOST_DIRECT", direct)
    s = make(300, seed=15, K=16)
    qel, qion = s.to_pt()
    qel["ff"] = np.random.default_rng(3).normal(size=(s.nel, 3))
    qion["ff"] = np.random.default_rng(4).normal(size=(s.nion, 3))
    p = T.params_for(s, precision="fp64", recip="spme")
    with T.Context(p, s.nel, s.nion) as c:
        c.upload_pt(qel, qion)
        a, b = np.zeros_like(qel), np.zeros_like(qion)
        a["id"], b["id"] = 5, 6
        c.download_pt(a, b)
        x, v, f, _ = c.download(x=True, v=True, f=True)
        c.upload(x=x[::-1].copy(), v=None, f=f * 2)
        x2, v2, f2, _ = c.download(x=True, v=True, f=True)
    for k in ("xx", "xv", "ff"):
        assert np.array_equal(a[k], qel[k]) and np.array_equal(b[k], qion[k])
    assert np.all(a["id"] == 5) and np.all(b["id"] == 6)
    assert np.array_equal(x, s.x) and np.array_equal(v, s.v)
    assert np.array_equal(x2, s.x[::-1]) and np.array_equal(v2, s.v) and np.array_equal(f2, 2 * f)


@pytest.mark.parametrize("direct", ["1", "0"])
@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_md_steps_records_equals_separate_calls(direct, precision, monkeypatch):
    """tcp_md_steps_records (records read, steps, records written, one wait)
    against tcp_upload x2 + tcp_md_steps + tcp_download x2 on the same records:
    bitwise, through both transfer paths; other record fields untouched."""
    monkeypatch.setenv("TCP_HOST_DIRECT", direct)
    s = make(600, seed=21, K=16)
    p = T.params_for(s, precision=precision, recip="spme")
    out = []
    for fused in (False, True):
        qel, qion = s.to_pt()
        qel["id"], qion["id"] = 3, 4
        with T.Context(p, s.nel, s.nion) as c:
            c.EWALD_SELF()
            c.set_flags(T.FLAG_ENERGY | T.FLAG_DETERMINISTIC)    # fixed-order sums: bitwise comparable
            c.upload_pt(qel, qion, fields=("xx", "xv"))
            c.force()
            c.download_pt(qel, qion, fields=("ff",))
            for _ in range(3):
                if fused:
                    e = c.md_steps_pt(s.dt, 2, qel, qion)
                else:
                    c.upload_pt(qel, qion)
                    e = c.md_steps(s.dt, 2)
                    c.download_pt(qel, qion)
        out.append((qel, qion, e))
    (a_el, a_ion, ea), (b_el, b_ion, eb) = out
    for k in ("xx", "xv", "ff"):
        assert np.array_equal(a_el[k], b_el[k]) and np.array_equal(a_ion[k], b_ion[k])
    assert np.all(b_el["id"] == 3) and np.all(b_ion["id"] == 4)
    assert ea == eb


def test_md_steps_records_rejects_bad_strides():
    s = make(64, seed=2, K=16)
    qel, qion = s.to_pt()
    p = T.params_for(s, precision="fp64", recip="spme")
    with T.Context(p, s.nel, s.nion) as c:
        c.EWALD_SELF()
        c.upload_pt(qel, qion)
        x0, _, _, _ = c.download(x=True, v=False, f=False)
        base = qel.ctypes.data
        off = {k: qel.dtype.fields[k][1] for k in ("xx", "xv", "ff")}
        ptr = [C.c_void_p(base + off[k]) for k in ("xx", "xv", "ff")]
        e = T.TcpEnergies()
        rc = c.lib.tcp_md_steps_records(c.h, s.dt, 1, *ptr, 20, None, None, None, 104, C.byref(e))
        assert rc == _abi.TCP_ERR_BAD_PARAM
        x1, _, _, _ = c.download(x=True, v=False, f=False)
    assert np.array_equal(x0, x1)                 # nothing ran


def test_errors():
    s = make(64, seed=14, K=16)
    p = T.params_for(s, precision="fp64", recip="spme")
    p.rc = 0.6 * s.box
    with T.Context(p, s.nel, s.nion) as c:
        with pytest.raises(T.TcpError) as ei:
            c.EWALD_SELF()
        assert ei.value.code == 2            # TCP_ERR_CUTOFF, force.f90:18-22
        with pytest.raises(T.TcpError) as ei:
            c.Force_direct_self()
        assert ei.value.code == 7            # TCP_ERR_STATE


def test_large_fp32c_rows_sample():
    """N = 65536 (the headline size): sampled rows of the real-space sum vs
    the oracle, and size-independent properties of the full sum."""
    s = T.make_config_system("n65536_spme128", seed=0)
    o = oracle.Oracle.from_system(s, ei="kelbg")
    rows = np.r_[0:256, 32768:33024]
    with ctx_for(s, precision="fp32c", ei="kelbg", recip="none") as c:
        c.Force_direct_self()
        _, _, f, _ = c.download(x=False, v=False, f=True)
    fo = np.concatenate([o.force_direct_rows(s.x, 0, 256)[0], o.force_direct_rows(s.x, 32768, 33024)[0]])
    assert oracle.rms_rel(f[rows], fo) < FP32_FORCE_RMS
    # ordered-pair sums without reactions: Newton's third law holds only to rounding
    assert np.linalg.norm(f.sum(0)) < 1e-6 * np.abs(f).sum()


@pytest.mark.parametrize("variant", list(range(19)))
@pytest.mark.parametrize("ei,n", [("kelbg", 2048), ("deutsch", 1536), ("kelbg", 1000)])
def test_fp32c_kernel_variants(monkeypatch, variant, ei, n):
    """Every real-space kernel the autotuner can pick (0 = ordered pairs,
    1 = scalar Newton-3, 2..18 = Newton-3 with packed FP32x2 arithmetic,
    6..16 and 18 with the degree-5 Ewald erfc, 12 and 13 with six
    i-particles per lane, 14, 15, 17 and 18 with two warps per CTA, 16 with
    one) against the oracle, including partial tiles."""
    monkeypatch.setenv("TCP_PAIR_VARIANT", str(variant))
    s = make(n, seed=30 + variant)
    o = oracle.Oracle.from_system(s, ei=ei)
    fo, uo = o.force_direct(s.x)
    with ctx_for(s, precision="fp32c", ei=ei, recip="none") as c:
        ur = c.Force_direct_self()
        _, _, f, _ = c.download(x=False, v=False, f=True)
        assert c.autotune_report()[0] == variant
    assert oracle.rms_rel(f, fo) < FP32_FORCE_RMS
    assert ur == pytest.approx(uo, rel=2e-5)


def test_autotuner_picks_a_timed_variant(monkeypatch):
    monkeypatch.delenv("TCP_PAIR_VARIANT", raising=False)
    s = make(8192, seed=40)
    with ctx_for(s, precision="fp32c", ei="kelbg", recip="none") as c:
        c.Force_direct_self()
        v, ms = c.autotune_report()
    assert 0 <= v <= 18
    assert ms[v] > 0 and ms[v] == min(m for m in ms if m > 0)


def test_grid_reserve_for_the_overlapped_reciprocal_chain(monkeypatch):
    """With SPME the autotuner also times the pair kernel with the reciprocal
    chain beside it for a few grid reserves and keeps the smallest within
    0.3 % of the fastest;
    TCP_PAIR_RESERVE forces one, and the forces do not depend on it (a
    Newton-3 variant is forced: at this size the ordered kernel can win)."""
    monkeypatch.setenv("TCP_PAIR_VARIANT", "10")
    monkeypatch.delenv("TCP_PAIR_RESERVE", raising=False)
    s = make(8192, seed=41, K=32, order=5)
    with ctx_for(s, precision="fp32c", ei="kelbg", recip="spme") as c:
        c.force()
        r, cand = c.overlap_report()
    assert set(cand) == {0, 16, 32, 64, 128, 256, 512}
    # the smallest reserve within 0.3 % of the fastest
    assert r in cand and cand[r] <= 1.003 * min(cand.values())
    assert all(cand[q] > 1.003 * min(cand.values()) for q in cand if q < r)
    forces = []
    for forced in ("0", "40"):
        monkeypatch.setenv("TCP_PAIR_RESERVE", forced)
        with ctx_for(s, precision="fp32c", ei="kelbg", recip="spme") as c:
            e = c.force()
            _, _, f, _ = c.download(x=False, v=False, f=True)
            assert c.overlap_report() == (int(forced), {})
        forces.append((f, e["Ur"]))
    assert oracle.rms_rel(forces[1][0], forces[0][0]) < 1e-6
    assert forces[1][1] == pytest.approx(forces[0][1], rel=1e-6)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_noncubic_box_and_mesh_uneven_species(precision):
    """Box (L, 1.1 L, 0.9 L), mesh (20, 16, 24), order 5, 600 electrons and 424
    ions: the ordered-pair FP32C kernel's general-box path and the spread's
    unequal mesh dimensions against the oracle."""
    rng = np.random.default_rng(77)
    nel, nion = 600, 424
    L = T.make_system(nel + nion, seed=1).box
    box = (L, 1.1 * L, 0.9 * L)
    x = (rng.random((nel + nion, 3)) - 0.5) * np.array(box)
    v = rng.normal(0.0, 0.1, size=(nel + nion, 3))
    rc = 0.45 * min(box)
    alpha = 3.1 / rc
    o = oracle.Oracle(nel, nion, box, rc, alpha=alpha, lambda_ei=0.5 * T.EPS, rs=0.5 * T.EPS, ei="kelbg",
                      K=(20, 16, 24), order=5)
    fo, uro, umo = o.force_total(x, recip="spme")
    s = T.make_system(nel + nion, seed=1)
    p = T.params_for(s, precision=precision, ei="kelbg", recip="spme")
    for d in range(3):
        p.box[d] = box[d]
    p.K[0], p.K[1], p.K[2] = 20, 16, 24
    p.order = 5
    p.rc = rc
    p.a = alpha
    p.lambda_ei = p.rs = 0.5 * T.EPS
    with T.Context(p, nel, nion) as c:
        c.EWALD_SELF()
        c.upload(x=x, v=v)
        e = c.force()
        _, _, f, _ = c.download(x=False, v=False, f=True)
    tol = 1e-10 if precision == "fp64" else FP32_FORCE_RMS
    assert oracle.rms_rel(f, fo) < tol
    assert e["Um"] == pytest.approx(umo, rel=1e-10 if precision == "fp64" else 1e-6)
    assert e["Ur"] == pytest.approx(uro, rel=1e-10 if precision == "fp64" else 2e-5)


@pytest.mark.parametrize("ei", ["deutsch", "kelbg", "coulomb"])
@pytest.mark.parametrize("nel,nion", [(1024, 1024), (700, 333), (1, 300), (257, 0)])
def test_fp64_newton3_vs_ordered(ei, nel, nion):
    """The FP64 Newton-3 kernel (default) against the ordered-pair FP64
    kernel (TCP_FLAG_DETERMINISTIC) and the oracle: partial i-tiles and
    j-subtiles, a single electron, one species only."""
    s = T.make_system(nel + nion, gamma=1.0, lam=0.5, seed=8, alpha_rc=3.1, K=16, order=4)
    s.nel, s.nion = nel, nion
    o = oracle.Oracle.from_system(s, ei=ei)
    fo, uo = o.force_direct(s.x)
    out = {}
    for det in (False, True):
        with ctx_for(s, precision="fp64", ei=ei, recip="none") as c:
            if det:
                c.set_flags(T.FLAG_ENERGY | T.FLAG_DETERMINISTIC)
            ur = c.Force_direct_self()
            _, _, f, _ = c.download(x=False, v=False, f=True)
        out[det] = (ur, f)
        assert ur == pytest.approx(uo, rel=FP64_REL, abs=1e-12)
        assert oracle.rms_rel(f, fo) < FP64_REL
    assert oracle.rms_rel(out[False][1], out[True][1]) < 1e-13
    assert out[False][0] == pytest.approx(out[True][0], rel=1e-13, abs=1e-13)


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_deterministic_flag_is_bitwise_reproducible(precision):
    """With TCP_FLAG_DETERMINISTIC two force evaluations of the same state give
    identical bits (ordered-pair kernels, fixed-order reductions, atomic-free
    SPME spread)."""
    s = make(3000, seed=9, K=24, order=5)
    with ctx_for(s, precision=precision, ei="kelbg", recip="spme") as c:
        c.set_flags(T.FLAG_ENERGY | T.FLAG_DETERMINISTIC)
        e1 = c.force()
        _, _, f1, _ = c.download(x=False, v=False, f=True)
        e2 = c.force()
        _, _, f2, _ = c.download(x=False, v=False, f=True)
    assert np.array_equal(f1, f2)
    assert e1["Ur"] == e2["Ur"] and e1["Um"] == e2["Um"]


@pytest.mark.parametrize("variant", [0, 1, 2, 10, 14, 16])
@pytest.mark.parametrize("r_over_lam", [1e-3, 1e-2, 0.1, 0.3, 0.49, 0.8, 2.0])
def test_kelbg_close_pair_accuracy(monkeypatch, variant, r_over_lam):
    """One electron and one ion at r = (1e-3 .. 2) lambda: the Kelbg e-i force
    and energy of the FP32C kernels (ordered, scalar and packed Newton-3)
    against the FP64 oracle.  Below lambda/2 the force numerator
    erfc(ar) + 2ar/sqrt(pi) e^{-a^2r^2} - e^{-r^2/lambda^2} is of order
    r^2/lambda^2 while each term is of order 1; the series form keeps the
    FP32 relative accuracy there."""
    monkeypatch.setenv("TCP_PAIR_VARIANT", str(variant))
    s = T.make_system(2, gamma=1.0, lam=0.5, seed=1, alpha_rc=3.1, K=8, order=4)
    assert s.nel == 1 and s.nion == 1
    lam = s.lambda_ei
    u = np.array([0.48, -0.6, 0.64])
    u /= np.linalg.norm(u)
    x = np.zeros((2, 3))
    x[1] = r_over_lam * lam * u
    o = oracle.Oracle.from_system(s, ei="kelbg")
    fo, uo = o.force_direct(x)
    with T.Context(T.params_for(s, precision="fp32c", ei="kelbg", recip="none"), 1, 1) as c:
        c.EWALD_SELF()
        c.upload(x=x, v=np.zeros((2, 3)))
        ur = c.Force_direct_self()
        _, _, f, _ = c.download(x=False, v=False, f=True)
    assert np.linalg.norm(f - fo) / np.linalg.norm(fo) < 2e-5
    assert ur == pytest.approx(uo, rel=2e-5, abs=1e-6 * abs(uo) + 1e-12)


@pytest.mark.parametrize("variant", [2, 4, 5, 10, 12, 13, 14, 15, 16, 17])
@pytest.mark.parametrize("nel,nion", [(1, 300), (257, 0), (700, 333), (1030, 2)])
def test_fp32c_newton3_ragged_species(monkeypatch, variant, nel, nion):
    """Packed Newton-3 variants with a single electron, one species only, and
    species counts that leave partial i-tiles and j-subtiles, against the
    oracle (Kelbg, real-space sum)."""
    monkeypatch.setenv("TCP_PAIR_VARIANT", str(variant))
    s = T.make_system(nel + nion, gamma=1.0, lam=0.5, seed=21, alpha_rc=3.1, K=16, order=4)
    s.nel, s.nion = nel, nion
    fo, uo = oracle.Oracle.from_system(s, ei="kelbg").force_direct(s.x)
    with ctx_for(s, precision="fp32c", ei="kelbg", recip="none") as c:
        ur = c.Force_direct_self()
        _, _, f, _ = c.download(x=False, v=False, f=True)
        assert c.autotune_report()[0] == variant
    assert oracle.rms_rel(f, fo) < FP32_FORCE_RMS
    assert ur == pytest.approx(uo, rel=2e-5, abs=1e-9)


def test_fp32c_with_fp64_reciprocal_chain(monkeypatch):
    """TCP_PREC_FP32C_R64: the FP32C real-space sum with the SPME chain
    (spread, transforms, influence, gather) in FP64.  Its reciprocal forces
    and Um are the FP64 context's (the same deterministic FP64 chain), its
    real-space forces the FP32C context's, and its whole step agrees with the
    oracle to the FP32C bound; the precision is fixed at tcp_create.  Both
    FP32C contexts run the same real-space variant (the autotuners could pick
    degree-5 and degree-6 erfc forms, whose Ur differ at the 1e-6 level)."""
    monkeypatch.setenv("TCP_PAIR_VARIANT", "17")   # n3_r4_u2_w2b8_x2
    s = make(2048, seed=44, K=32, order=5)
    comps = {}
    for prec in ("fp64", "fp32c", "fp32c_r64"):
        with ctx_for(s, precision=prec, ei="kelbg", recip="spme") as c:
            ur = c.Force_direct_self()
            _, _, fr, _ = c.download(x=False, v=False, f=True)
            um = c.Force_SPME4()
            _, _, _, frec = c.download(x=False, v=False, f=False, frec=True)
            e = c.force()
            _, _, ft, _ = c.download(x=False, v=False, f=True)
            if prec == "fp32c_r64":
                q = T.params_for(s, precision="fp32c", ei="kelbg", recip="spme")
                with pytest.raises(T.TcpError):
                    c.set_params(q)
                c.set_params(T.params_for(s, precision="fp32c_r64", ei="kelbg", recip="spme"))
        comps[prec] = dict(real=fr, ur=ur, recip=frec, um=um, total=ft, e=e)
    r64, f64, f32 = comps["fp32c_r64"], comps["fp64"], comps["fp32c"]
    assert oracle.rms_rel(r64["recip"], f64["recip"]) < 1e-13
    assert r64["um"] == pytest.approx(f64["um"], rel=1e-13)
    assert oracle.rms_rel(r64["real"], f32["real"]) < 1e-6
    assert r64["ur"] == pytest.approx(f32["ur"], rel=1e-6)
    fo, uro, umo = oracle.Oracle.from_system(s, ei="kelbg").force_total(s.x, recip="spme")
    assert oracle.rms_rel(r64["total"], fo) < FP32_FORCE_RMS
    assert r64["e"]["Um"] == pytest.approx(umo, rel=1e-10)


def test_charged_system_background_energy():
    """A system with net charge (40 electrons, 24 ions): Uo carries the
    neutralising-background energy -pi Q^2/(2 V alpha^2) exactly as the
    oracle's, and the FP64 Ewald total (Ur + Uo) eps + Um of the plain k-sum
    does not depend on alpha."""
    rng = np.random.default_rng(4)
    nel, nion, L = 40, 24, 20.0
    x = (rng.random((nel + nion, 3)) - 0.5) * L
    s = T.make_system(nel + nion, seed=1)
    totals = []
    for arc in (4.5, 5.0):
        p = T.params_for(s, precision="fp64", ei="coulomb", recip="ewald", nmax2=400)
        for d in range(3):
            p.box[d] = L
        p.rc = L / 2
        p.a = arc / p.rc
        o = oracle.Oracle(nel, nion, L, p.rc, alpha=p.a, ei="coulomb", K=0)
        with T.Context(p, nel, nion) as c:
            _, uo = c.EWALD_SELF()
            c.upload(x=x)
            e = c.force()
        assert uo == pytest.approx(o.Uo, rel=1e-14)
        totals.append(e["Epot"] + e["Um"])
    assert totals[0] == pytest.approx(totals[1], rel=1e-9)


def snap_to_grid(x, box):
    """Positions on the fixed-point grid of the FP32C kernels (2^32 points per
    box length), so that both the GPU and the FP64 oracle see the same
    separations up to FP64 rounding."""
    box = np.broadcast_to(np.asarray(box, dtype=np.float64), (3,))
    m = np.floor((x / box + 0.5) * 2.0 ** 32) % 2.0 ** 32
    return (m / 2.0 ** 32 - 0.5) * box


@pytest.mark.parametrize("rdf_variant", [0, 1, 2, 3])
def test_fp32c_newton3_rdf_histograms(monkeypatch, rdf_variant):
    """RDF counts of the packed Newton-3 forms (+2 per unique pair inside rc,
    force.f90:99-103) equal the FP64 oracle's bin for bin: pairs whose FP32
    r/dx or r^2 lies near a bin edge or rc are binned from the exact integer
    r^2 of their fixed-point separation.  Positions on the fixed-point grid,
    so both sides bin the same separations; forces and energy as without the
    histograms."""
    monkeypatch.setenv("TCP_PAIR_VARIANT", "10")
    monkeypatch.setenv("TCP_RDF_VARIANT", str(rdf_variant))
    s = make(4096, seed=13, K=16)
    s.x = snap_to_grid(s.x, s.box)
    o = oracle.Oracle.from_system(s, ei="kelbg")
    fo, uo, h = o.force_direct(s.x, rdf=True)
    with ctx_for(s, precision="fp32c", ei="kelbg", recip="none") as c:
        c.set_flags(T.FLAG_ENERGY | T.FLAG_RDF)
        ur = c.Force_direct_self()
        _, _, f, _ = c.download(x=False, v=False, f=True)
        rdf, _ = c.histograms(reset=True)
    assert np.array_equal(rdf, h)
    assert oracle.rms_rel(f, fo) < FP32_FORCE_RMS
    assert ur == pytest.approx(uo, rel=2e-5)


@pytest.mark.parametrize("precision", ["fp32c", "fp64"])
@pytest.mark.parametrize("box_kind", ["cubic", "noncubic"])
def test_ordered_rdf_histograms(precision, box_kind):
    """The ordered-pair kernels (TCP_FLAG_DETERMINISTIC; in FP32C the only
    kernel of non-cubic boxes) count +1 from each side of a pair, FP32C with
    the same exact binning as the Newton-3 forms: equal to the oracle's RDF.
    700 + 333 particles leave partial i-blocks, whose padding lanes must count
    nothing."""
    nel, nion = 700, 333
    s = make(nel + nion, seed=17, K=16)
    s.nel, s.nion = nel, nion
    box = (s.box, s.box, s.box) if box_kind == "cubic" else (s.box, 1.1 * s.box, 0.9 * s.box)
    rng = np.random.default_rng(3)
    x = snap_to_grid((rng.random((s.n, 3)) - 0.5) * np.array(box), box)
    rc = 0.45 * min(box)
    o = oracle.Oracle(nel, nion, box, rc, alpha=3.1 / rc, lambda_ei=s.lambda_ei, rs=s.lambda_ei, ei="deutsch",
                      K=16, order=4, rdf_dx=rc / T.NDIST)
    _, _, h = o.force_direct(x, rdf=True)
    p = T.params_for(s, precision=precision, ei="deutsch", recip="none", rdf_dx=rc / T.NDIST)
    for d in range(3):
        p.box[d] = box[d]
    p.rc = rc
    p.a = 3.1 / rc
    with T.Context(p, nel, nion) as c:
        c.set_flags(T.FLAG_ENERGY | T.FLAG_RDF | T.FLAG_DETERMINISTIC)
        c.EWALD_SELF()
        c.upload(x=x)
        c.Force_direct_self()
        rdf, _ = c.histograms(reset=True)
    assert np.array_equal(rdf, h)
