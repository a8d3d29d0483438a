"""Benchmark of the TCP_allpair force-and-integrate step on GB300.

Headline workload (the largest single-GPU configuration): N = 65,536
(32,768 electrons + 32,768 ions), Gamma = 1, Kelbg e-i lambda = 0.5 a,
Ewald alpha from erfc(alpha rc) = 1e-6 with rc = L/2, SPME 128^3 order 5,
NVE velocity Verlet, seeded synthetic inputs.  A "step" is one MD step
(first half kick + drift, SPME, all-pair real-space sum, net-force removal,
second half kick, energy and kinetic reductions).

value      pair-int/s = N(N-1)/2 * steps / time of the compensated-FP32 step,
           state resident in HBM, CUDA events per step on the library's stream,
           L2 flushed (2x L2 written) between timed steps.
e2e        the same metric through the C ABI with host PT records: every step
           reads x, v, f from the records, runs one step and writes x, v, f
           back (tcp_md_steps_records); `separate_calls` times the same work
           as tcp_upload x2 + tcp_md_steps + tcp_download x2.
fp64       the plain FP64 drop-in step at the same configuration.
recip_fp64_option
           the FP32C step with the whole SPME chain in FP64 (TCP_PREC_FP32C_R64).
roofline   the real-space pair kernel against the measured FP32 FFMA issue rate.
force_error / energy_error
           at the seeded start: RMS relative error of the real-space,
           reciprocal and total force and the largest per-particle error, and
           the relative errors of Ur, Um, Uo and Etot, FP32C against the FP64
           GPU path and every GPU path against the FP64 restatement (all rows).
nve_drift / nve_drift_fp64
           total-energy drift over 500 NVE steps, FP32C and FP64.
c2         the N = 16,384 isokinetic workload (Gamma 2, lambda 0.4 a, SPME
           64^3 order 4, rescale every 10 steps, 1000 steps): FP64 and FP32C
           step times, errors against the restatement, Etot difference.
batch      64 replicas (N log-uniform in [512, 8192]) in one persistent launch
           per step against looping one context per replica.
cpu_baseline / --impl reference
           the FP64 CPU restatement (oracle/, OpenMP on all host cores; the
           Fortran/MPI reference cannot be built on this machine): full MD steps
           (direct sum over all pairs, SPME, integrator).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import atexit
import json
import math
import os
import pathlib
import re
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "pair-int/s, steps/s @N=65536: FP32-comp vs FP64 on 1 GB300, ≤2e-6 force err"
WORKLOAD = "n65536_spme128"
EPS = 14.399644154020082      # eV*A, data.f90:21
# Source-level op recipe of the FP32C real-space kernels (pair.cu tile_f32,
# pair_n3.cu n3_pair/n3_item), Coulomb pair with energy, cubic box: 3 integer
# subtractions + 3 int->float conversions (minimum image), r^2 (3), cut-off
# test (1), r (1), rcp argument (1), exp argument (1), erfc polynomial
# (degree 6) and products (9), force numerator (1), 1/r mask select and r^-2
# weight (3), force accumulation (3), energy add (1) = 30 per ordered pair; the
# Newton-3 kernel adds the reaction accumulation (3) = 33 per unique pair.
# The Newton-3 variants named "_p5" evaluate a degree-5 erfc polynomial (one
# FFMA fewer): 32 per unique pair.  SFU: rsqrt, rcp, ex2 (3) per pair in all.
RECIPE_ORDERED = 30
RECIPE_N3 = 33
RECIPE_N3_P5 = 32
RECIPE_SFU_OPS = 3
SFU_RATE = 16.0 / 128.0       # SFU lanes per SM relative to FP32 lanes
REF_MAX_STEPS = 5             # full CPU steps timed by --impl reference


def log(*a):
    print(*a, file=sys.stderr, flush=True)


class Clocks:
    """nvidia-smi sampler running during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.proc = None
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.device = device

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
            return self
        # the timed region starts once the sampler writes (nvidia-smi takes a moment to start)
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 3.0 and self.proc.poll() is None:
            if pathlib.Path(self.f.name).stat().st_size > 0:
                break
            time.sleep(0.02)
        self.skip = pathlib.Path(self.f.name).read_text().count("\n")   # samples taken before the region
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.proc:
            return None
        self.f.flush()
        rows = [r.split(",") for r in pathlib.Path(self.f.name).read_text().splitlines() if r.strip()]
        rows = rows[getattr(self, "skip", 0):] or rows[-1:]
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for k, nm in enumerate(names):
                if len(r) > 5 + k and r[5 + k].strip().lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist  # plumbing only: barrier and max over ranks
        dist.init_process_group(backend="gloo")
    return world, rank, local, dist


def barrier(dist):
    if dist:
        dist.barrier()


def reduce_max(dist, x: float) -> float:
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(dist, x: float) -> float:
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def profile_traffic():
    """DRAM bytes per launch of the pair kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "pair_n3_kelbg_n65536.md"
    if not p.exists():
        return None
    m = re.search(r"dram_bytes_per_launch_full_size:\s*([0-9.eE+]+)", p.read_text())
    return float(m.group(1)) if m else None


# ---------------------------------------------------------------------------
# CPU leg: full MD steps of the FP64 restatement
def kinetic(s):
    """(1/2) sum m v^2 of the seeded start (eV), the same for every arm."""
    m = np.concatenate([np.full(s.nel, s.xm[0]), np.full(s.nion, s.xm[1])])
    return 0.5 * float(np.sum(m[:, None] * s.v * s.v))


def oracle_components(o, x):
    """Real-space, reciprocal and total forces (REMOVE_RIGIDMTN applied to the
    total, main.f90:141) and the energies of the FP64 restatement at x."""
    f_real, ur = o.force_direct(x)
    f_rec, um = o.force_spme(x)
    f_tot = f_real + f_rec
    f_tot -= f_tot.mean(axis=0)
    return dict(real=f_real, recip=f_rec, total=f_tot, Ur=ur, Um=um, Uo=o.Uo, Epot=(ur + o.Uo) * EPS)


def gpu_components(ctx):
    """The same quantities from a context at its current positions: the direct
    sum alone (tcp_force_direct), then the whole evaluation (tcp_force), whose
    reciprocal forces stay readable as frec."""
    ctx.Force_direct_self()
    _, _, f_real, _ = ctx.download(x=False, v=False, f=True)
    e = ctx.force()
    _, _, f_tot, f_rec = ctx.download(x=False, v=False, f=True, frec=True)
    return dict(real=f_real, recip=f_rec, total=f_tot, Ur=e["Ur"], Um=e["Um"], Uo=e["Uo"], Epot=e["Epot"])


def force_errors(a, ref):
    """RMS relative error of the real-space, reciprocal and total force, and the
    largest per-particle error of the total, relative to that particle's force
    and to the RMS force."""
    import oracle
    d = np.linalg.norm(a["total"] - ref["total"], axis=1)
    fr = np.linalg.norm(ref["total"], axis=1)
    rms = float(np.sqrt(np.mean(fr ** 2)))
    return {"real": oracle.rms_rel(a["real"], ref["real"]), "recip": oracle.rms_rel(a["recip"], ref["recip"]),
            "total": oracle.rms_rel(a["total"], ref["total"]),
            "max_particle_rel": float(np.max(d / np.maximum(fr, 1e-300))),
            "max_particle_over_rms": float(np.max(d) / rms)}


def energy_errors(a, ref, ekin):
    """Relative errors of Ur, Um, Uo and Etot = Ekin + Epot + Um (the ener files)."""
    def rel(x, y):
        return abs(x - y) / abs(y) if y != 0 else abs(x - y)
    et_a, et_r = ekin + a["Epot"] + a["Um"], ekin + ref["Epot"] + ref["Um"]
    return {"Ur": rel(a["Ur"], ref["Ur"]), "Um": rel(a["Um"], ref["Um"]), "Uo": rel(a["Uo"], ref["Uo"]),
            "Etot": rel(et_a, et_r)}


def cpu_steps(s, nsteps: int, threads: int, warmup: int = 0):
    """Full MD steps of the FP64 restatement (OpenMP on `threads` cores): the
    initial force evaluation (kept for the error figures), `warmup` untimed
    steps, then `nsteps` timed steps, each vverlet1 + direct sum over all
    pairs + SPME + vverlet2 (main.f90:81-153)."""
    import oracle
    o = oracle.Oracle.from_system(s, ei="kelbg", nthreads=threads)
    t0 = time.perf_counter()
    comp = oracle_components(o, s.x)
    t_first = time.perf_counter() - t0
    x, v, f = s.x.copy(), s.v.copy(), comp["total"].copy()
    for _ in range(warmup):
        o.md_step(x, v, f, s.dt)
    t0 = time.perf_counter()
    for _ in range(nsteps):
        o.md_step(x, v, f, s.dt)
    t_steps = time.perf_counter() - t0
    pairs = s.n * (s.n - 1) / 2
    t_step = t_steps / max(nsteps, 1)
    return dict(t_step=t_step, value=pairs / t_step, t_first=t_first, t_steps=t_steps, comp=comp)


def run_reference(args, world, rank, dist):
    """--impl reference: the CPU restatement (the reference itself cannot be built)."""
    if rank != 0:
        return 0
    import oracle
    from tcp_allpair_gb300.system import make_config_system
    oracle.build()
    s = make_config_system(WORKLOAD, seed=0)
    threads = os.cpu_count() or 1
    # a full step takes seconds on the host cores: at most REF_MAX_STEPS timed steps after one
    # untimed one, so that the arm ends within a minute whatever --steps asks for
    steps, warmup = max(1, min(args.steps, REF_MAX_STEPS)), min(args.warmup, 1)
    t0 = time.perf_counter()
    cs = cpu_steps(s, steps, threads, warmup=warmup)
    wall = time.perf_counter() - t0
    t_step = cs["t_step"]
    n = s.n
    value = n * (n - 1) / 2 / t_step
    sample = (f"{steps} full MD steps after {warmup} untimed one(s) ({args.steps} asked): direct sum over all "
              f"N(N-1)/2 pairs (FP64, OpenMP), SPME 128^3 p5, integrator")
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "pair-int/s", "n_gpus": args.gpus,
        "steps": steps, "warmup": warmup, "steps_requested": args.steps, "warmup_requested": args.warmup,
        "ms_per_step": t_step * 1e3, "steps_per_s": 1.0 / t_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded uniform positions (0.1a rejection), Maxwell-Boltzmann velocities",
        "config": config_dict(s),
        "reference_note": "the Fortran 90 + MPI + FFTE reference cannot be built here or on the GPU box "
                          "(no Fortran compiler, no MPI, FFTE not vendored); timed is the FP64 C restatement "
                          "of force.f90/vverlet.f90 in oracle/",
        "cpu_baseline": {"value": value, "unit": "pair-int/s", "cores": threads, "kind": "port", "sample": sample,
                         "timed_s": cs["t_steps"]},
        "e2e": {"value": value, "unit": "pair-int/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "wall_s": wall,
    }
    print(json.dumps(out))
    return 0


def config_dict(s):
    return {"workload": "n65536_spme128_kelbg_nve", "N": s.n, "nel": s.nel, "nion": s.nion, "gamma": 1.0,
            "lambda_ei_over_a": 0.5, "ei_model": "kelbg", "box_A": s.box, "rc": "L/2",
            "ewald_alpha_rc": s.alpha * s.rc, "spme_mesh": s.K, "spline_order": s.order, "ensemble": "NVE",
            "dt_over_wpe": 0.01, "units": "reference (A, eV, amu, 10.18 fs)",
            "precision": "FP32 pair arithmetic with compensated accumulation; SPME on a compensated-FP32 mesh "
                         "with FP32 transforms; FP64 integration and reductions",
            "l2": "flushed between timed steps (a 2x L2 buffer is written outside the timed spans)"}


def nve_drift(T, p, s, nsteps, device, precision):
    """Relative total-energy drift over nsteps NVE steps from the seeded start,
    Etot = (mv2el + mv2ion)/2 + Epot + Um as in the ener files, sampled ten times."""
    with T.Context(p, s.nel, s.nion, device=device) as c:
        c.EWALD_SELF()
        c.upload(x=s.x, v=s.v)
        c.force()

        def etot(e):
            return 0.5 * (e["mv2el"] + e["mv2ion"]) + e["Epot"] + e["Um"]

        e = c.md_steps(s.dt, 1)
        E0 = etot(e)
        worst, done = 0.0, 1
        every = max(1, nsteps // 10)
        t0 = time.perf_counter()
        while done < nsteps:
            k = min(every, nsteps - done)
            e = c.md_steps(s.dt, k)
            done += k
            worst = max(worst, abs(etot(e) - E0) / abs(E0))
        wall = time.perf_counter() - t0
    return {"steps": nsteps, "E_step1_eV": E0, "rel_drift_end": abs(etot(e) - E0) / abs(E0),
            "rel_drift_max_sampled": worst, "sampled_every": every, "precision": precision,
            "wall_s": wall}


def run_c2(T, args, device, threads):
    """The N = 16,384 workload: Gamma 2, lambda 0.4 a, SPME 64^3 order 4, the
    isokinetic rescale to T = 0.5 every 10 steps (vverlet.f90:301-372), run
    `args.c2_steps` steps in FP64 and in FP32C from the same start.  Reports
    both step times, the force and energy errors of both at the start against
    the FP64 restatement, and the FP32C - FP64 total-energy difference along
    the run (the thermostat does not conserve energy, so no drift figure)."""
    import oracle
    from tcp_allpair_gb300.system import make_config_system
    s = make_config_system("n16384_spme64", seed=0)
    o = oracle.Oracle.from_system(s, ei="kelbg", nthreads=threads)
    ref = oracle_components(o, s.x)
    ek = kinetic(s)
    pairs = s.n * (s.n - 1) / 2
    out = {"workload": "n16384_spme64_kelbg_isokin10", "N": s.n, "gamma": 2.0, "lambda_ei_over_a": 0.4,
           "spme_mesh": s.K, "spline_order": s.order, "thermostat": "isokin every 10 steps to T = 0.5",
           "steps": args.c2_steps}
    traj = {}
    for prec in ("fp64", "fp32c"):
        p = T.params_for(s, precision=prec, ei="kelbg", recip="spme", thermo="isokin", thermo_period=10)
        with T.Context(p, s.nel, s.nion, device=device) as c:
            c.EWALD_SELF()
            c.upload(x=s.x, v=s.v)
            comp = gpu_components(c)
            t = c.time_steps(s.dt, 20, flush_l2=True)        # device time of one step
            kernel = c.variant_name(c.autotune_report()[0]) if prec == "fp32c" else "pair_n3_f64_kernel"
            reserve = c.overlap_report() if prec == "fp32c" else None
            recip_alone = c.time_component(1, 5)
            pair_alone = c.time_component(0, 5)
            # the run itself from the seeded start, Etot sampled every tenth of it
            c.upload(x=s.x, v=s.v)
            c.force()
            every = max(1, args.c2_steps // 10)
            et = []
            t0 = time.perf_counter()
            for _ in range(args.c2_steps // every):
                e = c.md_steps(s.dt, every)
                et.append(0.5 * (e["mv2el"] + e["mv2ion"]) + e["Epot"] + e["Um"])
            wall = time.perf_counter() - t0
        ms = t["step"] / t["nsteps"]
        out[prec] = {"ms_per_step": ms, "value": pairs / (ms * 1e-3), "run_wall_s": wall,
                     "breakdown_ms_per_step": {k: t[k] / t["nsteps"] for k in ("vverlet1", "pair", "recip",
                                                                              "epilogue")},
                     "pair_kernel": kernel, "pair_alone_ms": pair_alone, "recip_alone_ms": recip_alone,
                     "grid_reserve": reserve[0] if reserve else None,
                     "reserve_ms": reserve[1] if reserve else None,
                     "force_error_vs_oracle": force_errors(comp, ref),
                     "energy_error_vs_oracle": energy_errors(comp, ref, ek)}
        traj[prec] = np.array(et)
    out["speedup_fp32c_over_fp64"] = out["fp64"]["ms_per_step"] / out["fp32c"]["ms_per_step"]
    d = np.abs(traj["fp32c"] - traj["fp64"]) / np.abs(traj["fp64"])
    out["etot_fp32c_vs_fp64"] = {"rel_diff_max_sampled": float(d.max()), "rel_diff_end": float(d[-1]),
                                 "sampled_every": max(1, args.c2_steps // 10)}
    return out


def run_batch_leg(T, args, device):
    """The batched-replica workload: 64 independent systems (N log-uniform in
    [512, 8192], Gamma log-uniform in [0.1, 10], lambda uniform in [0.2a, 0.8a],
    own box, alpha and SPME mesh) stepped together in one graph per step,
    against looping one context per replica over the same steps."""
    from tcp_allpair_gb300.system import make_batch_systems
    ss = make_batch_systems(args.batch_reps, seed=0)
    params = [T.params_for(s, precision="fp32c", ei="kelbg", recip="spme") for s in ss]
    pairs = sum(s.n * (s.n - 1) / 2 for s in ss)
    dt = ss[0].dt
    with T.Batch(params, [s.nel for s in ss], [s.nion for s in ss], device=device) as b:
        b.EWALD_SELF()
        for r, s in enumerate(ss):
            b.upload(r, x=s.x, v=s.v)
        b.force()
        bvar, bms = b.autotune_report()
        bres, bres_ms = b.overlap_report()
        bname = b.variant_name(bvar)
        b_names = [b.variant_name(v) for v in range(len(bms))]
        b.md_steps(dt, args.warmup)
        chain_alone = b.time_component(1, 10)
        pair_alone = b.time_component(0, 10)
        tb = b.time_steps(dt, args.steps, flush_l2=True)
        ms_batch = tb["step"] / tb["nsteps"]
        phases = {k: round(tb[k] / tb["nsteps"], 4) for k in ("vverlet1", "recip", "pair", "epilogue")}
    ms_loop = None
    ctxs = []
    for p_, s in zip(params, ss if args.batch_loop else []):
        c = T.Context(p_, s.nel, s.nion, device=device)
        c.EWALD_SELF()
        c.upload(x=s.x, v=s.v)
        c.force()
        c.md_steps(dt, args.warmup)
        ctxs.append(c)
    if ctxs:
        t0 = time.perf_counter()
        for _ in range(args.steps):
            for c in ctxs:
                c.lib.tcp_md_steps(c.h, dt, 1, None)
        for c in ctxs:
            c.md_steps(dt, 0)          # synchronise every stream
        ms_loop = (time.perf_counter() - t0) * 1e3 / args.steps
    for c in ctxs:
        c.close()
    # the batched pair launch against the FFMA peak
    peak = T.fp32_peak(device) * 1e12
    pair_ms = pair_alone
    recipe = RECIPE_N3_P5 if bname.endswith("_p5") else RECIPE_N3
    roof = {"bound": "fp32", "kernel": f"pair_n3_kernel batched (variant {bvar}: {bname})",
            "recipe": f"{recipe} FP32/ALU-pipe ops + {RECIPE_SFU_OPS} SFU ops per unique pair",
            "pair_kernel_alone_ms": pair_ms, "peak": peak / 1e12, "unit": "Top/s",
            "achieved": recipe * pairs / (pair_ms * 1e-3) / 1e12,
            "frac_alone": recipe * pairs / (pair_ms * 1e-3) / peak,
            "note": "the batched pair launch alone, mean of 10 launches (no chains beside it); "
                    "replicas of 256-4096 particles per species have many masked diagonal items"}
    return {"metric": "aggregate pair-int/s, batched replicas", "workload": f"batch{len(ss)}_n512-8192",
            "value": pairs / (ms_batch * 1e-3), "unit": "pair-int/s", "ms_per_step": ms_batch,
            "loop_single_contexts": {"value": pairs / (ms_loop * 1e-3), "ms_per_step": ms_loop} if ms_loop else None,
            "speedup_batch_over_loop": ms_loop / ms_batch if ms_loop else None, "replicas": len(ss),
            "particles": sum(s.n for s in ss), "steps": args.steps, "warmup": args.warmup,
            "l2": "flushed before each timed step", "phases_ms": phases,
            "alone_ms": {"pair": round(pair_alone, 4), "spme_chains": round(chain_alone, 4)},
            "batch_variant": int(bvar),
            "batch_variant_ms": {b_names[v]: round(float(x), 4) for v, x in enumerate(bms) if x > 0},
            "grid_reserve": bres, "reserve_ms": {k: round(v, 4) for k, v in bres_ms.items()},
            "roofline": roof}


def run_gpu(args, world, rank, local, dist):
    import oracle
    import tcp_allpair_gb300 as T
    from tcp_allpair_gb300.system import make_config_system

    # one autotuning per workload for all contexts of this run, in a file private to the
    # run: the e2e context runs the kernel and grid reserve that the timed context chose
    if "TCP_AUTOTUNE_CACHE" not in os.environ:
        fd, cache = tempfile.mkstemp(prefix="tcp_autotune_", suffix=".txt")
        os.close(fd)
        os.environ["TCP_AUTOTUNE_CACHE"] = cache
        atexit.register(lambda: os.path.exists(cache) and os.unlink(cache))
    s = make_config_system(WORKLOAD, seed=rank)
    n = s.n
    pairs = n * (n - 1) / 2
    ek = kinetic(s)
    p32 = T.params_for(s, precision="fp32c", ei="kelbg", recip="spme", thermo="notemp")
    p64 = T.params_for(s, precision="fp64", ei="kelbg", recip="spme", thermo="notemp")
    pr64 = T.params_for(s, precision="fp32c_r64", ei="kelbg", recip="spme", thermo="notemp")
    ctx = T.Context(p32, s.nel, s.nion, device=local)
    ctx.EWALD_SELF()
    ctx.upload(x=s.x, v=s.v)
    e0 = ctx.force()                        # initial forces (restart-style start, main.f90:49-54)
    tune = ctx.autotune_report()
    ctx_name = ctx.variant_name(tune[0])
    ctx_names = [ctx.variant_name(k) for k in range(len(tune[1]))]
    reserve, reserve_ms = ctx.overlap_report()
    comp32 = gpu_components(ctx)
    ctx.upload(x=s.x, v=s.v)
    ctx.force()

    ctx64 = T.Context(p64, s.nel, s.nion, device=local)
    ctx64.EWALD_SELF()
    ctx64.upload(x=s.x, v=s.v)
    comp64 = gpu_components(ctx64)
    ctx64.upload(x=s.x, v=s.v)
    ctx64.force()

    # warm-up, then the timed steps (device-resident)
    ctx.md_steps(s.dt, args.warmup)
    launches0 = ctx.launch_count()
    barrier(dist)
    with Clocks(local) as clk:
        t = ctx.time_steps(s.dt, args.steps, flush_l2=True)
    launches = ctx.launch_count() - launches0
    barrier(dist)
    step_ms = t["step"] / t["nsteps"]
    step_ms_max = reduce_max(dist, step_ms)
    value = reduce_sum(dist, pairs) * args.steps / (step_ms_max * args.steps * 1e-3)
    pair_ms = t["pair"] / t["nsteps"]
    # the reciprocal chain by itself (it runs concurrently with the pair kernel
    # inside a step, on a second stream)
    recip_alone_ms = ctx.time_component(1, 5)
    # the same steps with the RDF histograms accumulated in the pair sum, as the
    # reference's Force_direct_self does in every call (force.f90:99-103)
    ctx.set_flags(T.FLAG_ENERGY | T.FLAG_RDF)
    ctx.md_steps(s.dt, args.warmup)
    t_rdf = ctx.time_steps(s.dt, args.steps, flush_l2=True)
    ctx.set_flags(T.FLAG_ENERGY)
    rdf_step = {"ms_per_step": t_rdf["step"] / t_rdf["nsteps"],
                "value": pairs / (t_rdf["step"] / t_rdf["nsteps"] * 1e-3),
                "pair_kernel_ms": t_rdf["pair"] / t_rdf["nsteps"],
                "note": "TCP_FLAG_RDF: the ee/ei/ii pair-distance histograms of force.f90:99-103 binned in "
                        "the pair kernel at every step (the headline steps leave them off, as the library "
                        "does unless the caller asks)"}

    # FP64 drop-in step (few steps: FP64 issue rate of GB300 is ~1/64 of FP32)
    ctx64.md_steps(s.dt, 1)
    t64 = ctx64.time_steps(s.dt, args.fp64_steps, flush_l2=True)
    step64_ms = t64["step"] / t64["nsteps"]
    ctx64.close()

    # the FP32C step with the whole reciprocal chain in FP64 (TCP_PREC_FP32C_R64)
    with T.Context(pr64, s.nel, s.nion, device=local) as cr:
        cr.EWALD_SELF()
        cr.upload(x=s.x, v=s.v)
        comp_r64 = gpu_components(cr)
        cr.upload(x=s.x, v=s.v)
        cr.force()
        cr.md_steps(s.dt, args.warmup)
        tr = cr.time_steps(s.dt, args.steps, flush_l2=True)
        recip64_alone_ms = cr.time_component(1, 5)
        r64_reserve, r64_reserve_ms = cr.overlap_report()
    r64_ms = tr["step"] / tr["nsteps"]
    recip_fp64 = {"ms_per_step": r64_ms, "value": pairs / (r64_ms * 1e-3),
                  "pair_kernel_ms": tr["pair"] / tr["nsteps"], "recip_concurrent_wall": tr["recip"] / tr["nsteps"],
                  "recip_alone_ms": recip64_alone_ms, "step_time_ratio_vs_fp32c_recip": r64_ms / step_ms,
                  "grid_reserve": r64_reserve, "reserve_ms": {k: round(v, 4) for k, v in r64_reserve_ms.items()},
                  "note": "TCP_PREC_FP32C_R64: the FP32C real-space sum with the SPME spread, transforms, "
                          "influence multiply and gather in FP64, on the second stream beside the pair kernel"}

    # NVE energy drift over the headline run length (500 steps), FP32C and FP64
    drift = drift64 = None
    if rank == 0:
        if args.nve_steps > 0:
            drift = nve_drift(T, p32, s, args.nve_steps, local, "fp32c")
        if args.nve_fp64_steps > 0:
            drift64 = nve_drift(T, p64, s, args.nve_fp64_steps, local, "fp64")

    # e2e through the C ABI with host PT records
    qel, qion = s.to_pt()
    ctx_e = T.Context(p32, s.nel, s.nion, device=local)
    ctx_e.EWALD_SELF()
    ctx_e.upload_pt(qel, qion, fields=("xx", "xv"))
    ctx_e.force()
    ctx_e.download_pt(qel, qion)
    ctx_e.md_steps(s.dt, 1)
    barrier(dist)
    ph = [0.0, 0.0, 0.0]                       # host wall time of upload, step, download
    for _ in range(args.steps):                # the three calls, each timed
        t0 = time.perf_counter()
        ctx_e.upload_pt(qel, qion)
        t1 = time.perf_counter()
        ctx_e.md_steps(s.dt, 1)
        t2 = time.perf_counter()
        ctx_e.download_pt(qel, qion)
        t3 = time.perf_counter()
        ph[0] += t1 - t0
        ph[1] += t2 - t1
        ph[2] += t3 - t2
    te_sep = reduce_max(dist, sum(ph))
    barrier(dist)
    te0 = time.perf_counter()                  # the headline e2e: one call per step on the records
    for _ in range(args.steps):
        ctx_e.md_steps_pt(s.dt, 1, qel, qion)
    te = time.perf_counter() - te0
    te = reduce_max(dist, te)
    e2e_tuning = {"variant": ctx_e.variant_name(ctx_e.autotune_report()[0]), "grid_reserve": ctx_e.overlap_report()[0]}
    ctx_e.close()
    e2e_value = reduce_sum(dist, pairs) * args.steps / te
    e2e_sep_value = reduce_sum(dist, pairs) * args.steps / te_sep
    stride = qel.strides[0]
    h2d = sum((len(a) - 1) * stride + 72 for a in (qel, qion) if len(a))   # span xx(1)..ff(3) per species
    d2h = n * 3 * 3 * 8

    # roofline of the pair kernel (live timing inside the timed steps)
    peak = T.fp32_peak(local) * 1e12            # FFMA/s = lane instructions/s
    variant, variant_ms = tune
    if variant >= 1:
        recipe = RECIPE_N3_P5 if ctx_name.endswith("_p5") else RECIPE_N3
        units, kname = float(n) * (n - 1) / 2, f"pair_n3_kernel (Newton-3 variant {variant}: {ctx_name})"
        runit = "unique pair"
    else:
        units, recipe, kname = float(n) * (n - 1), RECIPE_ORDERED, "pair_fp32c_kernel (ordered pairs)"
        runit = "ordered pair"
    achieved = recipe * units / (pair_ms * 1e-3)
    sfu_frac = RECIPE_SFU_OPS * units / (pair_ms * 1e-3) / (peak * SFU_RATE)
    traffic = profile_traffic()
    roof = {"bound": "fp32", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "Top/s",
            "frac": achieved / peak, "traffic": traffic,
            "kernel": kname,
            "autotune_ms": {f"{k} {ctx_names[k]}": round(x, 4) for k, x in enumerate(variant_ms.tolist()) if x > 0},
            "recipe": f"{recipe} FP32/ALU-pipe ops + {RECIPE_SFU_OPS} SFU ops per {runit}",
            "peak_source": "measured FFMA issue rate (tcp_fp32_peak) on this GPU, not MEASURED_PEAKS.json "
                           "(which has HBM and bf16 only)",
            "sfu_frac": sfu_frac, "pair_kernel_ms": pair_ms,
            # the same launch timed by the autotuner alone (no reciprocal chain beside it)
            "pair_kernel_alone_ms": float(variant_ms[variant]),
            "frac_alone": recipe * units / (float(variant_ms[variant]) * 1e-3) / peak if variant_ms[variant] > 0 else None,
            "grid_reserve": reserve, "reserve_ms": reserve_ms}

    # CPU baseline (rank 0, N = 1 only): full steps of the FP64 restatement, whose
    # initial evaluation is also the reference of the force and energy errors
    cpu = None
    ferr = {"bound_total_rms": 2e-6,
            "definition": "RMS relative sqrt(sum|F-F_ref|^2 / sum|F_ref|^2) per component over all particles; "
                          "max_particle_rel = max_i |dF_i|/|F_ref_i|, max_particle_over_rms = max_i |dF_i| / "
                          "RMS|F_ref|; total includes REMOVE_RIGIDMTN",
            "fp32c_vs_fp64_gpu": force_errors(comp32, comp64)}
    eerr = {"fp32c_vs_fp64_gpu": energy_errors(comp32, comp64, ek)}
    c2 = batch = None
    if rank == 0 and world == 1:
        threads = os.cpu_count() or 1
        if args.cpu_steps > 0:          # --cpu-steps 0: no CPU leg (profiling runs)
            cs = cpu_steps(s, args.cpu_steps, threads)
            ref = cs["comp"]
            cpu = {"value": cs["value"], "unit": "pair-int/s", "cores": threads, "kind": "port",
                   "sample": f"{args.cpu_steps} full MD steps of the FP64 restatement (direct sum over all "
                             f"N(N-1)/2 pairs with OpenMP, SPME 128^3 p5, integrator), {cs['t_steps']:.1f} s timed",
                   "ms_per_step": cs["t_step"] * 1e3}
            ferr["fp32c_vs_oracle"] = force_errors(comp32, ref)
            ferr["fp64_gpu_vs_oracle"] = force_errors(comp64, ref)
            ferr["fp32c_r64_vs_oracle"] = force_errors(comp_r64, ref)
            eerr["fp32c_vs_oracle"] = energy_errors(comp32, ref, ek)
            eerr["fp64_gpu_vs_oracle"] = energy_errors(comp64, ref, ek)
            eerr["fp32c_r64_vs_oracle"] = energy_errors(comp_r64, ref, ek)
        if args.c2_steps > 0:
            c2 = run_c2(T, args, local, threads)
        if args.batch_reps > 0:
            batch = run_batch_leg(T, args, local)

    ctx.close()
    clocks = clk.summary()
    out = {
        "metric": METRIC, "value": value, "unit": "pair-int/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": step_ms_max, "steps_per_s": 1e3 / step_ms_max,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded uniform positions (0.1a rejection), Maxwell-Boltzmann velocities",
        "config": config_dict(s),
        "breakdown_ms_per_step": {"vverlet1": t["vverlet1"] / t["nsteps"], "pair": pair_ms,
                                  "recip_concurrent_wall": t["recip"] / t["nsteps"],
                                  "recip_alone": recip_alone_ms, "epilogue": t["epilogue"] / t["nsteps"],
                                  "note": "the SPME chain runs on a second stream beside the pair kernel; "
                                          "recip_concurrent_wall is its span inside the step, recip_alone "
                                          "the same chain timed by itself"},
        "fp64": {"ms_per_step": step64_ms, "value": pairs / (step64_ms * 1e-3), "steps": args.fp64_steps,
                 "speedup_fp32c_over_fp64": step64_ms / step_ms},
        "recip_fp64_option": recip_fp64,
        "rdf_every_step": rdf_step,
        "force_error": ferr,
        "energy_error": eerr,
        "energies_initial": {"Ur": e0["Ur"], "Um": e0["Um"], "Uo": e0["Uo"]},
        "nve_drift": drift,
        "nve_drift_fp64": drift64,
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "pair-int/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "ms_per_step": te / args.steps * 1e3,
                "path": "tcp_md_steps_records(1): PT records x,v,f read, one step, x,v,f written back, "
                        "pageable host memory",
                "tuning": e2e_tuning,
                "separate_calls": {"ms_per_step": te_sep / args.steps * 1e3,
                                   "value": e2e_sep_value,
                                   "host_ms_per_step": {"upload": ph[0] / args.steps * 1e3,
                                                        "md_steps": ph[1] / args.steps * 1e3,
                                                        "download": ph[2] / args.steps * 1e3},
                                   "path": "tcp_upload x2 + tcp_md_steps(1) + tcp_download x2"}},
        "c2": c2,
        "batch": batch,
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(out))
    return 0


def run_pair_only(args):
    """Launch the real-space pair kernel alone on an N-particle version of the
    headline system (profiling target: `ncu --clock-control none -k regex:pair_
    -c 1 ... python bench.py --pair-only N`); with --rdf, the form that also
    bins the RDF histograms."""
    import tcp_allpair_gb300 as T
    n = args.pair_only
    s = T.make_system(n, gamma=1.0, lam=0.5, seed=0, ewald_rel_err=1e-6, K=64, order=5)
    p = T.params_for(s, precision=args.precision, ei="kelbg", recip="none")
    with T.Context(p, s.nel, s.nion) as c:
        c.EWALD_SELF()
        c.upload(x=s.x, v=s.v)
        if args.rdf:
            c.set_flags(T.FLAG_ENERGY | T.FLAG_RDF)
        for _ in range(3):
            c.Force_direct_self()
        ms = c.time_component(0, 5)
    print(json.dumps({"pair_only": n, "precision": args.precision, "rdf": bool(args.rdf), "pair_kernel_ms": ms}))
    return 0


def run_recip_only(args):
    """Launch the SPME chain alone on the `--config` system (default the
    headline one) with N particles (profiling target: `ncu --clock-control none
    -k regex:spme -c 3 ... python bench.py --recip-only N`)."""
    import tcp_allpair_gb300 as T
    from tcp_allpair_gb300.system import make_config_system
    s = make_config_system(args.config, n=args.recip_only)
    p = T.params_for(s, precision=args.precision, ei="kelbg", recip="spme")
    with T.Context(p, s.nel, s.nion) as c:
        c.EWALD_SELF()
        c.upload(x=s.x, v=s.v)
        for _ in range(3):
            c.Force_SPME4()
        ms = c.time_component(1, 5)
    print(json.dumps({"recip_only": args.recip_only, "precision": args.precision, "spme_ms": ms}))
    return 0


def run_batch(args):
    """--batch: the batched-replica leg alone."""
    import tcp_allpair_gb300 as T
    print(json.dumps(run_batch_leg(T, args, 0)))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--cpu-steps", type=int, default=3, help="full CPU steps of the cpu_baseline leg")
    ap.add_argument("--nve-steps", type=int, default=500, help="FP32C NVE energy-drift run (0: skip)")
    ap.add_argument("--nve-fp64-steps", type=int, default=500, help="FP64 NVE energy-drift run (0: skip)")
    ap.add_argument("--c2-steps", type=int, default=1000, help="N = 16,384 isokinetic run (0: skip)")
    ap.add_argument("--pair-only", type=int, default=0, help="profile target: pair kernel alone at this N")
    ap.add_argument("--rdf", action="store_true", help="with --pair-only: the form that bins the RDF histograms")
    ap.add_argument("--recip-only", type=int, default=0, help="profile target: SPME chain alone at this N")
    ap.add_argument("--precision", default="fp32c", choices=["fp32c", "fp64"])
    ap.add_argument("--config", default="n65536_spme128", help="named workload of --recip-only")
    ap.add_argument("--batch", action="store_true", help="batched-replica workload instead of the headline")
    ap.add_argument("--batch-reps", type=int, default=64, help="replicas of the batched leg (0: skip)")
    ap.add_argument("--no-batch-loop", dest="batch_loop", action="store_false",
                    help="batched leg without the loop of one context per replica it is compared with")
    args = ap.parse_args()
    if args.batch:
        return run_batch(args)
    if args.pair_only:
        return run_pair_only(args)
    if args.recip_only:
        return run_recip_only(args)
    args.warmup = max(args.warmup, 3)
    world, rank, local, dist = dist_setup()
    if args.impl == "reference":
        rc = run_reference(args, world, rank, dist)
    else:
        rc = run_gpu(args, world, rank, local, dist)
    if dist:
        dist.destroy_process_group()
    return rc


if __name__ == "__main__":
    sys.exit(main())
