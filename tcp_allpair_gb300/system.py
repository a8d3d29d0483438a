"""Seeded two-component plasma systems and the named workload configurations.

A system is built in reduced units (length a = Wigner-Seitz radius, energy
e^2/a, electron mass 1) and converted to the reference's units (data.f90:21-22:
Angstrom, eV, amu, time in tps = 10.18 fs) by scaling every length with
eps = 14.399644154020082, so that e^2/a = 1 eV:

    x_ref = eps x_red,  t_ref = eps t_red,  v_ref = v_red,  T_ref[eV] = T_red,
    F_ref[eV/A] = F_red / eps,  masses in amu (m_e = 1, m_i = 1836).

Positions are uniform in [-L/2, L/2)^3 with minimum-image separations of at
least 0.1 a (rejection and redraw), velocities Maxwell-Boltzmann per species,
mean removed per species and rescaled to the exact target temperature (so the
total momentum is zero).  The particle arrays follow the reference ordering:
electrons first, then ions (main.f90:358-378).
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

EPS = 14.399644154020082      # data.f90:21
TPS = 10.180505306645389      # data.f90:22
NDIST = 500                   # data.f90:16

# PT record of data.f90:32-35 (id, xx(3), xv(3), ff(3), vi(3)) as laid out by
# gfortran/ifort: 4-byte id, 4 bytes of padding, 12 doubles -> 104 bytes.
PT_DTYPE = np.dtype([("id", "<i4"), ("_pad", "<i4"), ("xx", "<f8", 3), ("xv", "<f8", 3),
                     ("ff", "<f8", 3), ("vi", "<f8", 3)])
assert PT_DTYPE.itemsize == 104


def box_length_reduced(n: int) -> float:
    """L = (4 pi N / 3)^(1/3) in units of the Wigner-Seitz radius."""
    return (4.0 * math.pi * n / 3.0) ** (1.0 / 3.0)


@dataclasses.dataclass
class System:
    """Particle state and parameters in reference units."""
    nel: int
    nion: int
    box: float
    x: np.ndarray            # (N, 3) positions [A], wrapped into [-L/2, L/2)
    v: np.ndarray            # (N, 3) velocities [A / tps-unit]
    xm: tuple                # masses [amu]
    q: tuple                 # charges [e]
    Te: float                # target temperatures [eV]
    Ti: float
    rc: float                # real-space cut-off [A]
    alpha: float             # Ewald alpha [1/A]
    lambda_ei: float         # Kelbg / Deutsch length [A]
    dt: float                # time step [tps units]
    K: int = 0
    order: int = 4
    seed: int = 0

    @property
    def n(self) -> int:
        return self.nel + self.nion

    def to_pt(self):
        """(qel, qion) structured arrays with the PT layout of data.f90:32-35."""
        qel = np.zeros(self.nel, dtype=PT_DTYPE)
        qion = np.zeros(self.nion, dtype=PT_DTYPE)
        qel["xx"] = self.x[: self.nel]
        qel["xv"] = self.v[: self.nel]
        qel["id"] = np.arange(1, self.nel + 1)
        qion["xx"] = self.x[self.nel:]
        qion["xv"] = self.v[self.nel:]
        qion["id"] = np.arange(1, self.nion + 1)
        return qel, qion


def _wrap(x: np.ndarray, L: float) -> np.ndarray:
    """x - L * DNINT(x/L) (vverlet.f90:153): round half away from zero."""
    t = x / L
    return x - L * np.where(t >= 0.0, np.floor(t + 0.5), np.ceil(t - 0.5))


def uniform_positions(n: int, L: float, min_sep: float, rng: np.random.Generator) -> np.ndarray:
    """Uniform positions in [-L/2, L/2)^3 with all minimum-image pair distances
    >= min_sep (redraw one particle of every violating pair until none is left)."""
    from scipy.spatial import cKDTree

    u = rng.random((n, 3)) * L
    for _ in range(1000):
        u = np.mod(u, L)
        tree = cKDTree(u, boxsize=L)
        pairs = tree.query_pairs(min_sep, output_type="ndarray")
        if len(pairs) == 0:
            return u - 0.5 * L
        bad = np.unique(pairs[:, 1])
        u[bad] = rng.random((len(bad), 3)) * L
    raise RuntimeError("could not place particles with the requested separation")


def mb_velocities(count: int, T: float, m: float, rng: np.random.Generator) -> np.ndarray:
    """Maxwell-Boltzmann velocities, mean removed, rescaled so that
    sum m v^2 / (3 count) == T exactly (the normalisation of init.f90:53-60)."""
    if count == 0:
        return np.zeros((0, 3))
    v = rng.normal(0.0, math.sqrt(T / m), size=(count, 3))
    if count > 1:               # (a lone particle keeps its direction: removing the mean would stop it)
        v -= v.mean(axis=0)
    T0 = m * np.sum(v * v) / (3.0 * count)
    return v * math.sqrt(T / T0)


def make_system(n: int, gamma: float = 1.0, lam: float = 0.5, seed: int = 0,
                alpha_rc: float | None = None, ewald_rel_err: float | None = None,
                K: int = 0, order: int = 4, mass_ion: float = 1836.0,
                min_sep: float = 0.1, nel: int | None = None, T: float | None = None) -> System:
    """Build a seeded system in reference units.

    n      total particle count (n/2 electrons q=-1 m=1, n/2 ions q=+1 m=mass_ion)
    gamma  coupling: T = 1/gamma in e^2/a (= eV)
    lam    e-i length (Kelbg lambda / Deutsch rs) in units of a
    alpha  Ewald alpha: alpha_rc / rc when alpha_rc is given; from erfc(alpha rc)
           = ewald_rel_err when that is given; otherwise the reference's 3.1/rc
           (force.f90:23)
    """
    from scipy.special import erfcinv

    rng = np.random.default_rng(seed)
    nel = n // 2 if nel is None else nel
    nion = n - nel
    Lr = box_length_reduced(n)
    xr = uniform_positions(n, Lr, min_sep, rng)
    Tr = (1.0 / gamma) if T is None else T
    v = np.concatenate([mb_velocities(nel, Tr, 1.0, rng), mb_velocities(nion, Tr, mass_ion, rng)])
    L = EPS * Lr
    rc = 0.5 * L
    if alpha_rc is not None:
        alpha = alpha_rc / rc
    elif ewald_rel_err is not None:
        alpha = float(erfcinv(ewald_rel_err)) / rc
    else:
        alpha = 3.1 / rc
    dt = EPS * 0.01 / math.sqrt(3.0)        # 0.01 / omega_pe, omega_pe = sqrt(3)
    x = _wrap(EPS * xr, L)
    return System(nel=nel, nion=nion, box=L, x=x, v=v, xm=(1.0, mass_ion), q=(-1.0, 1.0),
                  Te=Tr, Ti=Tr, rc=rc, alpha=alpha, lambda_ei=EPS * lam, dt=dt, K=K,
                  order=order, seed=seed)


# Named workloads (the five benchmark configurations of the benchmark spec).
CONFIGS = {
    # Plain method, FP64, CPU: N=1024, Gamma=1, lambda=0.5, alpha=5.6/L, |k|<=8*2pi/L, 200 NVE steps
    "n1024_ewald": dict(n=1024, gamma=1.0, lam=0.5, alpha_rc=2.8, K=0, order=4, steps=200,
                        recip="ewald", nmax2=64, thermo="notemp", ei="kelbg"),
    # N=16384, Gamma=2, lambda=0.4, SPME 64^3 order 4, rescale to T=0.5 every 10 steps, 1000 steps
    "n16384_spme64": dict(n=16384, gamma=2.0, lam=0.4, alpha_rc=3.1, K=64, order=4, steps=1000,
                          recip="spme", thermo="isokin", period=10, ei="kelbg"),
    # headline: N=65536, Gamma=1, lambda=0.5, SPME 128^3 order 5, alpha for 1e-6 error, 500 NVE steps
    "n65536_spme128": dict(n=65536, gamma=1.0, lam=0.5, ewald_rel_err=1e-6, K=128, order=5,
                           steps=500, recip="spme", thermo="notemp", ei="kelbg"),
    # differentiation: N=4096, Gamma=1, lambda=0.5
    "n4096_adjoint": dict(n=4096, gamma=1.0, lam=0.5, alpha_rc=3.1, K=32, order=4, steps=200,
                          recip="spme", thermo="notemp", ei="kelbg"),
}


def make_config_system(name: str, seed: int = 0, n: int | None = None) -> System:
    c = CONFIGS[name]
    kw = dict(gamma=c["gamma"], lam=c["lam"], seed=seed, K=c.get("K", 0), order=c.get("order", 4))
    if "alpha_rc" in c:
        kw["alpha_rc"] = c["alpha_rc"]
    if "ewald_rel_err" in c:
        kw["ewald_rel_err"] = c["ewald_rel_err"]
    return make_system(n if n is not None else c["n"], **kw)


def make_batch_systems(nrep: int = 64, seed: int = 0, nmin: int = 512, nmax: int = 8192):
    """The batched-replica workload: N log-uniform in [nmin, nmax] (equal electrons
    and ions), Gamma log-uniform in [0.1, 10], lambda_ei uniform in [0.2a, 0.8a],
    alpha rc = 3.1 (force.f90:23), SPME order 4 on a 32^3 / 48^3 / 64^3 mesh
    chosen by N; replica r is seeded with seed + r."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(nrep):
        n = int(round(math.exp(rng.uniform(math.log(nmin), math.log(nmax)) ) / 2)) * 2
        gamma = math.exp(rng.uniform(math.log(0.1), math.log(10.0)))
        lam = rng.uniform(0.2, 0.8)
        K = 32 if n < 2048 else (48 if n < 4096 else 64)
        out.append(make_system(n, gamma=gamma, lam=lam, seed=seed + r, alpha_rc=3.1, K=K, order=4))
    return out
