"""Batched replicas (tcp_batch_*) against one context per replica and the oracle."""
import numpy as np
import pytest

import oracle
import tcp_allpair_gb300 as T

pytestmark = pytest.mark.gpu


def systems():
    spec = [(700, 1.0, 0.5, 16), (1024, 0.3, 0.3, 24), (1538, 5.0, 0.7, 32), (512, 2.0, 0.4, 16), (2050, 1.0, 0.6, 24)]
    return [T.make_system(n, gamma=g, lam=l, seed=50 + k, alpha_rc=3.1, K=K, order=4)
            for k, (n, g, l, K) in enumerate(spec)]


def same_erfc_kernels(monkeypatch):
    """Pin the batched and the single-system real-space kernel to the same form
    (R = 4, 2 warps per CTA, degree-5 erfc): the autotuners may otherwise pick a
    degree-5 erfc variant on one side and a degree-6 one on the other, whose
    energies differ at the 1e-6 level."""
    monkeypatch.setenv("TCP_BATCH_VARIANT", "13")   # b_r4_u2_w2b8_x2_p5
    monkeypatch.setenv("TCP_PAIR_VARIANT", "14")    # n3_r4_u2_w2b8_x2_p5


def test_batch_force_matches_single_contexts_and_oracle(monkeypatch):
    same_erfc_kernels(monkeypatch)
    ss = systems()
    params = [T.params_for(s, precision="fp32c", ei="kelbg", recip="spme") for s in ss]
    with T.Batch(params, [s.nel for s in ss], [s.nion for s in ss]) as b:
        uo = b.EWALD_SELF()
        for r, s in enumerate(ss):
            b.upload(r, x=s.x, v=s.v)
        eb = b.force()
        fb = [b.download(r, x=False, v=False)[2] for r in range(len(ss))]
    for r, s in enumerate(ss):
        with T.Context(params[r], s.nel, s.nion) as c:
            c.EWALD_SELF()
            c.upload(x=s.x, v=s.v)
            e = c.force()
            _, _, f, _ = c.download(x=False, v=False, f=True)
        assert oracle.rms_rel(fb[r], f) < 1e-6
        assert eb[r]["Ur"] == pytest.approx(e["Ur"], rel=1e-6)
        assert eb[r]["Um"] == pytest.approx(e["Um"], rel=1e-6)
        assert uo[r] == pytest.approx(e["Uo"], rel=1e-14)
        o = oracle.Oracle.from_system(s, ei="kelbg")
        fo, uro, umo = o.force_total(s.x)
        assert oracle.rms_rel(fb[r], fo) < 2e-6


def test_batch_md_steps_match_single_contexts(monkeypatch):
    same_erfc_kernels(monkeypatch)
    ss = systems()
    params = [T.params_for(s, precision="fp32c", ei="kelbg", recip="spme", thermo=th)
              for s, th in zip(ss, ["notemp", "isokin", "berend", "notemp", "isokin"])]
    with T.Batch(params, [s.nel for s in ss], [s.nion for s in ss]) as b:
        b.EWALD_SELF()
        for r, s in enumerate(ss):
            b.upload(r, x=s.x, v=s.v)
        b.force()
        eb = b.md_steps(ss[0].dt, 5)
        xb = [b.download(r, v=False, f=False)[0] for r in range(len(ss))]
    for r, s in enumerate(ss):
        with T.Context(params[r], s.nel, s.nion) as c:
            c.EWALD_SELF()
            c.upload(x=s.x, v=s.v)
            c.force()
            e = c.md_steps(s.dt, 5)
            x, _, _, _ = c.download(v=False, f=False)
        assert np.max(np.abs(xb[r] - x)) < 1e-6 * s.box
        assert eb[r]["mv2el"] == pytest.approx(e["mv2el"], rel=1e-5)
        assert eb[r]["Epot"] == pytest.approx(e["Epot"], rel=1e-5)


def test_batch_rejects_unsupported():
    s = systems()[0]
    p = T.params_for(s, precision="fp64", recip="spme")
    with pytest.raises(T.TcpError):
        T.Batch([p], [s.nel], [s.nion])


@pytest.mark.parametrize("variant", list(range(14)))
def test_batch_pair_variants_match_oracle(monkeypatch, variant):
    """Every batched real-space variant (TCP_BATCH_VARIANT) against the oracle's
    total force and the energies."""
    monkeypatch.setenv("TCP_BATCH_VARIANT", str(variant))
    ss = systems()[:3]
    params = [T.params_for(s, precision="fp32c", ei="kelbg", recip="spme") for s in ss]
    with T.Batch(params, [s.nel for s in ss], [s.nion for s in ss]) as b:
        b.EWALD_SELF()
        for r, s in enumerate(ss):
            b.upload(r, x=s.x, v=s.v)
        eb = b.force()
        chosen, _ = b.autotune_report()
        name = b.variant_name(chosen)
        fb = [b.download(r, x=False, v=False)[2] for r in range(len(ss))]
    assert chosen == variant and name.startswith("b_r")
    for r, s in enumerate(ss):
        fo, uro, umo = oracle.Oracle.from_system(s, ei="kelbg").force_total(s.x)
        assert oracle.rms_rel(fb[r], fo) < 2e-6
        assert eb[r]["Ur"] == pytest.approx(uro, rel=2e-5)


def test_batch_degree5_erfc_needs_every_replica(monkeypatch):
    """The degree-5 erfc variants are tuned and forced only when every
    replica's alpha rc is within the fit's range; one replica beyond it keeps
    the whole batch on the degree-6 variants."""
    ss = systems()[:2]
    ss.append(T.make_system(600, gamma=1.0, lam=0.5, seed=77, alpha_rc=3.8, K=16, order=4))
    params = [T.params_for(s, precision="fp32c", ei="kelbg", recip="spme") for s in ss]

    def run():
        with T.Batch(params, [s.nel for s in ss], [s.nion for s in ss]) as b:
            b.EWALD_SELF()
            for r, s in enumerate(ss):
                b.upload(r, x=s.x, v=s.v)
            eb = b.force()
            chosen, ms = b.autotune_report()
            fb = [b.download(r, x=False, v=False)[2] for r in range(len(ss))]
            return chosen, b.variant_name(chosen), ms, eb, fb

    monkeypatch.delenv("TCP_BATCH_VARIANT", raising=False)
    chosen, name, ms, _, _ = run()
    assert not name.endswith("_p5")
    assert ms[12] == 0 and ms[13] == 0 and all(m > 0 for m in ms[:12])
    monkeypatch.setenv("TCP_BATCH_VARIANT", "13")
    chosen, name, _, eb, fb = run()
    assert chosen == 0
    for r, s in enumerate(ss):
        fo, uro, _ = oracle.Oracle.from_system(s, ei="kelbg").force_total(s.x)
        assert oracle.rms_rel(fb[r], fo) < 2e-6
        assert eb[r]["Ur"] == pytest.approx(uro, rel=2e-5)


def test_batch_grid_reserve_and_rejoin(monkeypatch):
    """The batch autotuner times the batched pair launch with the SPME chains
    beside it for several grid reserves (the reserved CTAs rejoin the launch
    after the chains) and keeps the smallest within 0.3 % of the fastest;
    forced reserves give the same forces and energies.  The variant is fixed:
    the degree-5 and degree-6 erfc variants, which the autotuner may choose
    between from one run to the next, differ in Ur at the 1e-6 level."""
    monkeypatch.delenv("TCP_BATCH_RESERVE", raising=False)
    monkeypatch.setenv("TCP_BATCH_VARIANT", "12")
    ss = systems()
    params = [T.params_for(s, precision="fp32c", ei="kelbg", recip="spme") for s in ss]

    def run():
        with T.Batch(params, [s.nel for s in ss], [s.nion for s in ss]) as b:
            b.EWALD_SELF()
            for r, s in enumerate(ss):
                b.upload(r, x=s.x, v=s.v)
            e = b.force()
            f = [b.download(r, x=False, v=False)[2] for r in range(len(ss))]
            b.md_steps(ss[0].dt, 3)
            x = [b.download(r, v=False, f=False)[0] for r in range(len(ss))]
            return e, f, x, b.overlap_report()

    e0, f0, x0, (r, cand) = run()
    assert set(cand) == {0, 16, 32, 64, 128, 256, 512}
    assert r in cand and cand[r] <= 1.003 * min(cand.values())
    for forced in ("0", "512"):
        monkeypatch.setenv("TCP_BATCH_RESERVE", forced)
        e, f, x, (rr, _) = run()
        assert rr == int(forced)
        for k in range(len(ss)):
            assert oracle.rms_rel(f[k], f0[k]) < 1e-6
            assert e[k]["Ur"] == pytest.approx(e0[k]["Ur"], rel=1e-6)
            assert e[k]["Um"] == pytest.approx(e0[k]["Um"], rel=1e-6)
            assert np.max(np.abs(x[k] - x0[k])) < 1e-6 * ss[k].box


def test_batch_time_steps_phases(monkeypatch):
    """tcp_batch_time_steps: per-step event marks inside the step graph, with
    and without the L2 flush; the phases nest inside the step and the state
    advances by the steps timed."""
    monkeypatch.setenv("TCP_BATCH_VARIANT", "12")
    ss = systems()[:3]
    params = [T.params_for(s, precision="fp32c", ei="kelbg", recip="spme") for s in ss]
    with T.Batch(params, [s.nel for s in ss], [s.nion for s in ss]) as b:
        b.EWALD_SELF()
        for r, s in enumerate(ss):
            b.upload(r, x=s.x, v=s.v)
        b.force()
        x0 = b.download(0, v=False, f=False)[0]
        for flush in (True, False):
            t = b.time_steps(ss[0].dt, 4, flush_l2=flush)
            assert t["nsteps"] == 4
            assert all(t[k] > 0 for k in ("step", "vverlet1", "recip", "pair", "epilogue"))
            assert t["pair"] < t["step"] and t["recip"] < t["step"]
            assert t["vverlet1"] + max(t["pair"], t["recip"]) + t["epilogue"] <= t["step"] * 1.001
        x1 = b.download(0, v=False, f=False)[0]
        pair_ms, chain_ms = b.time_component(0, 3), b.time_component(1, 3)
        assert pair_ms > 0 and chain_ms > 0
        with pytest.raises(T.TcpError):
            b.time_component(2, 3)
        assert np.array_equal(b.download(0, v=False, f=False)[0], x1)   # timing leaves the state alone
    with T.Batch(params, [s.nel for s in ss], [s.nion for s in ss]) as b:
        b.EWALD_SELF()
        for r, s in enumerate(ss):
            b.upload(r, x=s.x, v=s.v)
        b.force()
        b.md_steps(ss[0].dt, 1 + 4 + 1 + 4)   # time_steps builds its graph with one step first
        x2 = b.download(0, v=False, f=False)[0]
    assert np.max(np.abs(x1 - x2)) < 1e-9 * ss[0].box
    assert np.max(np.abs(x1 - x0)) > 0
