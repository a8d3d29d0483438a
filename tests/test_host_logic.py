"""Host-side logic without a GPU: seeded inputs, the reference file formats,
the named workloads, and the multi-process reductions of bench.py over
torch.distributed (gloo, two ranks on 127.0.0.1)."""
import math
import multiprocessing as mp
import os
import socket
import sys

import numpy as np
import pytest
from scipy.special import erfc

import tcp_allpair_gb300 as T
from tcp_allpair_gb300 import refio
from tcp_allpair_gb300.system import CONFIGS, EPS, make_batch_systems, make_config_system

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_seeded_system_properties():
    s = T.make_system(512, gamma=2.0, lam=0.4, seed=3, alpha_rc=3.1, K=16)
    a = EPS                                                   # Wigner-Seitz radius in A
    assert s.box == pytest.approx(EPS * (4 * math.pi * 512 / 3) ** (1 / 3))
    assert np.all(s.x >= -s.box / 2) and np.all(s.x < s.box / 2)
    d = s.x[:, None, :] - s.x[None, :, :]
    d -= s.box * np.round(d / s.box)
    r = np.sqrt((d ** 2).sum(-1)) + np.eye(s.n) * 1e9
    assert r.min() >= 0.1 * a * (1 - 1e-12)                   # 0.1 a rejection
    for sl, m in ((slice(0, s.nel), 1.0), (slice(s.nel, s.n), 1836.0)):
        v = s.v[sl]
        assert np.allclose(v.sum(0), 0.0, atol=1e-12)          # zero momentum per species
        assert m * (v ** 2).sum() / (3 * len(v)) == pytest.approx(0.5, rel=1e-12)   # T = 1/Gamma
    assert s.dt == pytest.approx(EPS * 0.01 / math.sqrt(3.0))
    assert T.make_system(512, seed=3).x.tobytes() == T.make_system(512, seed=3).x.tobytes()


def test_headline_alpha_gives_1e6_ewald_error():
    s = make_config_system("n65536_spme128", n=1024)
    assert erfc(s.alpha * s.rc) == pytest.approx(1e-6, rel=1e-9)
    assert CONFIGS["n65536_spme128"]["K"] == 128 and CONFIGS["n65536_spme128"]["order"] == 5


def test_batch_workload_distribution():
    ss = make_batch_systems(64, seed=0)
    ns = np.array([s.n for s in ss])
    assert len(ss) == 64 and np.all(ns % 2 == 0) and ns.min() >= 512 and ns.max() <= 8192
    gam = np.array([1.0 / s.Te for s in ss])
    assert gam.min() >= 0.1 - 1e-12 and gam.max() <= 10.0 + 1e-12
    lam = np.array([s.lambda_ei / EPS for s in ss])
    assert lam.min() >= 0.2 and lam.max() <= 0.8
    assert set(s.K for s in ss) <= {32, 48, 64}


def test_restart_file_round_trip(tmp_path):
    s = T.make_system(64, seed=5)
    f = np.random.default_rng(1).normal(size=(s.n, 3))
    refio.write_restart_xyz(tmp_path / "REST01.xyz", s.x, s.v, f, s.nel)
    x, v, ff, ids = refio.read_rest(tmp_path / "REST01.xyz")
    assert np.array_equal(x, s.x) and np.array_equal(v, s.v) and np.array_equal(ff, f)
    assert list(ids[: s.nel]) == list(range(1, s.nel + 1)) and ids[s.nel] == 1


def _free_port():
    with socket.socket() as so:
        so.bind(("127.0.0.1", 0))
        return so.getsockname()[1]


def _rank_main(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    w, r, local, dist = bench.dist_setup()
    bench.barrier(dist)
    mx = bench.reduce_max(dist, float(rank + 1))
    sm = bench.reduce_sum(dist, float(rank + 1))
    dist.destroy_process_group()
    q.put((r, w, mx, sm))


def test_bench_reductions_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == [(0, 2, 2.0, 3.0), (1, 2, 2.0, 3.0)]


def test_reference_arm_line(monkeypatch, capsys):
    """bench.py --impl reference: full MD steps of the CPU restatement, at
    most five timed whatever --steps asks, and the JSON keys the reference
    line carries (the workload shrunk to 1,024 particles to stay quick)."""
    import argparse
    import json

    import bench
    from tcp_allpair_gb300 import system

    small = make_config_system("n65536_spme128", n=1024)
    small.K = 16
    monkeypatch.setattr(system, "make_config_system", lambda name, seed=0, n=None: small)
    args = argparse.Namespace(steps=100, warmup=5, gpus=1)
    assert bench.run_reference(args, 1, 0, None) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["steps"] == bench.REF_MAX_STEPS and line["warmup"] == 1
    assert line["steps_requested"] == 100 and line["unit"] == "pair-int/s" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": "pair-int/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    assert line["config"]["workload"] == "n65536_spme128_kelbg_nve"
