"""Failure detection without a GPU fault: host-side injected failures (device
allocation, cuFFT plan) and one bounded device wait made to run out (CTA 0 of
the Newton-3 kernel never issues its first subtile copy, TCP_INJECT_FAULT=
tile_wait): each call reports its status code, and the context (or a new one)
keeps working afterwards."""
import numpy as np
import pytest

import oracle
import tcp_allpair_gb300 as T
from tcp_allpair_gb300._abi import TCP_ERR_CUFFT, TCP_ERR_NOMEM, TCP_ERR_TIMEOUT

pytestmark = pytest.mark.gpu


def make(n=2048, seed=41):
    return T.make_system(n, gamma=1.0, lam=0.5, seed=seed, alpha_rc=3.1, K=16, order=4)


def test_injected_allocation_failure(monkeypatch):
    s = make()
    monkeypatch.setenv("TCP_INJECT_FAULT", "alloc")
    with pytest.raises(T.TcpError) as e:
        T.Context(T.params_for(s, precision="fp32c"), s.nel, s.nion)
    assert e.value.code == TCP_ERR_NOMEM
    monkeypatch.delenv("TCP_INJECT_FAULT")
    with T.Context(T.params_for(s, precision="fp32c"), s.nel, s.nion) as c:
        c.EWALD_SELF()


def test_injected_cufft_plan_failure(monkeypatch):
    s = make()
    c = T.Context(T.params_for(s, precision="fp64", recip="spme"), s.nel, s.nion)
    monkeypatch.setenv("TCP_INJECT_FAULT", "cufft_plan")
    with pytest.raises(T.TcpError) as e:
        c.EWALD_SELF()
    assert e.value.code == TCP_ERR_CUFFT
    c.close()
    monkeypatch.delenv("TCP_INJECT_FAULT")
    with T.Context(T.params_for(s, precision="fp64", recip="spme"), s.nel, s.nion) as c2:
        c2.EWALD_SELF()
        c2.upload(x=s.x, v=s.v)
        assert np.isfinite(c2.force()["Epot"])


def test_tile_wait_timeout_is_reported_and_context_recovers(monkeypatch):
    s = make(4096, seed=42)
    monkeypatch.setenv("TCP_PAIR_VARIANT", "2")          # the Newton-3 kernel, no autotuning launches
    p = T.params_for(s, precision="fp32c", ei="kelbg", recip="none")
    fo, uo = oracle.Oracle.from_system(s, ei="kelbg").force_direct(s.x)
    with T.Context(p, s.nel, s.nion) as c:
        c.EWALD_SELF()
        c.upload(x=s.x, v=s.v)
        monkeypatch.setenv("TCP_INJECT_FAULT", "tile_wait")
        with pytest.raises(T.TcpError) as e:
            c.Force_direct_self()
        assert e.value.code == TCP_ERR_TIMEOUT
        monkeypatch.delenv("TCP_INJECT_FAULT")
        ur = c.Force_direct_self()
        _, _, f, _ = c.download(x=False, v=False, f=True)
    assert oracle.rms_rel(f, fo) < 2e-6
    assert ur == pytest.approx(uo, rel=2e-5)
