"""tcp_drive: the main.f90 loop on the C ABI, fed the reference's tcp.prm /
restart.xyz and checked file by file (ener*.dat, RESTnn.xyz, RDFnnn.dat,
VDFnnn.dat) against an oracle replay of main.f90:81-168 and result.f90."""
import math
import subprocess

import numpy as np
import pytest

import oracle
import tcp_allpair_gb300 as T
from tcp_allpair_gb300 import _build, refio
from tcp_allpair_gb300.system import TPS

pytestmark = pytest.mark.gpu


def replay(s, o, x, v, f, nsteps, ndump, nsamp, nrest):
    """main.f90:81-168 with the oracle (NOTEMP, SPME order 4, Deutsch e-i)."""
    ener, rdfs, vdfs, rests = [], [], [], []
    rdf = np.zeros((3, 501))
    vdf = np.zeros((2, 501))
    for k in range(1, nsteps + 1):
        o.vverlet1(x, v, f, s.dt)
        fn, ur, um, h = o.force_total(x, recip="spme", rdf=True)
        f[:] = fn
        rdf += h
        me, mi, hv = o.vverlet2(v, f, s.dt, vdf=True)
        vdf += hv
        epot = (ur + o.Uo) * T.EPS
        if k % ndump == 0:
            rdfs.append(rdf.copy())
            vdfs.append(vdf.copy())
            rdf[:] = 0
            vdf[:] = 0
        if k % nsamp == 0:
            ener.append([k * s.dt * TPS, me / (3 * s.nel), mi / (3 * s.nion), epot + um,
                         0.5 * (me + mi) + epot + um])
        if k % nrest == 0:
            rests.append((x.copy(), v.copy(), f.copy()))
    return np.array(ener), rdfs, vdfs, rests


def test_tcp_drive_against_oracle_replay(tmp_path):
    _build.build()
    s = T.make_system(256, gamma=1.0, lam=0.5, seed=17, alpha_rc=3.1, K=16, order=4)
    o = oracle.Oracle.from_system(s, ei="deutsch")
    x, v = s.x.copy(), s.v.copy()
    f, _, _ = o.force_total(x)
    dt_fs = s.dt * TPS
    refio.write_tcp_prm(tmp_path / "tcp.prm", s, tmax_fs=20 * dt_fs, trest_fs=10 * dt_fs, tdump_fs=10 * dt_fs,
                        tsamp_fs=5 * dt_fs, thermo="NOTEMP", rest="ON")
    refio.write_restart_xyz(tmp_path / "restart.xyz", x, v, f, s.nel)
    r = subprocess.run([str(_build.DRIVE), "--precision", "fp64", str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr

    ener, rdfs, vdfs, rests = replay(s, o, x, v, f, 20, 10, 5, 10)
    got = np.concatenate([refio.read_ener(tmp_path / "ener00.dat"), refio.read_ener(tmp_path / "ener01.dat")])
    assert got.shape == (4, 5)
    assert np.allclose(got, ener, rtol=2e-8, atol=0)                  # ES15.8 rounding
    gx, gv, gf, ids = refio.read_rest(tmp_path / "REST02.xyz")
    rx, rv, rf = rests[1]
    assert np.allclose(gx, rx, rtol=1e-6, atol=1e-6 * s.box)          # ES14.6 rounding
    assert np.allclose(gv, rv, rtol=1e-6, atol=1e-12)
    assert list(ids[:3]) == [1, 2, 3]
    # DUMP normalisation, result.f90:244-262
    tab = refio.read_rdf(tmp_path / "RDF002.dat")
    V = s.box ** 3
    dx = s.rc / 500
    i = np.arange(1, 501)
    shell = i ** 3 - (i - 1) ** 3
    dv_ee = s.nel ** 2 * 10 * dx ** 3 * 4 * math.pi / 3 / V
    assert np.allclose(tab[:, 1], rdfs[1][0, :500] / dv_ee / shell, rtol=1e-6, atol=0)
    vtab = refio.read_rdf(tmp_path / "VDF002.dat")
    assert np.allclose(vtab[:, 1], vdfs[1][0, :500] / 10, rtol=1e-6, atol=0)
