"""Reference file formats: writers for tcp.prm / input.xyz / restart.xyz (read
by main.f90:221-441 and by tcp_drive) and readers for what result.f90 and
tcp_drive write (ener*.dat, RESTnn.xyz, RDFnnn.dat, VDFnnn.dat).

All quantities are in the reference's units (A, eV, amu, fs in the files).
"""
from __future__ import annotations

import pathlib

import numpy as np

from .system import TPS, System


def write_tcp_prm(path, sys: System, *, tmax_fs, trest_fs, tdump_fs, tsamp_fs, thermo="NOTEMP", tau=1.0,
                  alpha_lgv=0.0, rest="ON", trace="OFF", dx=None, K=None):
    """tcp.prm in the record order of main.f90:227-291 (one dummy line before each group)."""
    dt_fs = sys.dt * TPS
    dx = dx if dx is not None else sys.rc / 500
    K = K if K is not None else sys.K
    lines = [
        "TCP input",
        "time: tmax trest tdump tsamp dt (fs)",
        f"{tmax_fs!r} {trest_fs!r} {tdump_fs!r} {tsamp_fs!r} {dt_fs!r}",
        "box",
        f"{sys.box!r} {sys.box!r} {sys.box!r}",
        "temperature",
        f"{sys.Te!r}",
        f"{sys.Ti!r}",
        "particles",
        f"{sys.nel}",
        f"{sys.nion}",
        "cutoff",
        f"{sys.rc!r}",
        "rs",
        f"{sys.lambda_ei!r}",
        "mass",
        f"{sys.xm[0]!r}",
        f"{sys.xm[1]!r}",
        "charge",
        f"{sys.q[0]!r}",
        f"{sys.q[1]!r}",
        "thermostat",
        f"{thermo}",
        f"{tau!r} {alpha_lgv!r}",
        "restart",
        f"{rest} {trace}",
        "rdf",
        f"{dx!r} {dx!r} {dx!r}",
        "fft",
        f"{K} {K} {K}",
    ]
    pathlib.Path(path).write_text("\n".join(lines) + "\n")


def write_restart_xyz(path, x, v, f, nel, ids=None):
    """restart.xyz as read by main.f90:389-440: name x y z vx vy vz fx fy fz id."""
    n = len(x)
    ids = ids if ids is not None else np.r_[np.arange(1, nel + 1), np.arange(1, n - nel + 1)]
    rows = [f"{n}", "frame = 0 energy = 0"]
    for i in range(n):
        name = "Cu" if i < nel else "C"
        vals = " ".join(repr(float(a)) for a in (*x[i], *v[i], *f[i]))
        rows.append(f"{name} {vals} {int(ids[i])}")
    pathlib.Path(path).write_text("\n".join(rows) + "\n")


def write_input_xyz(path, x, nel, ids=None):
    """input.xyz as read by main.f90:353-378: name x y z id."""
    n = len(x)
    ids = ids if ids is not None else np.r_[np.arange(1, nel + 1), np.arange(1, n - nel + 1)]
    rows = [f"{n}", "frame = 0"]
    for i in range(n):
        rows.append(f"{'Cu' if i < nel else 'C'} {x[i][0]!r} {x[i][1]!r} {x[i][2]!r} {int(ids[i])}")
    pathlib.Path(path).write_text("\n".join(rows) + "\n")


def _table(path):
    rows = [r.split() for r in pathlib.Path(path).read_text().splitlines() if r.strip() and not r.startswith("#")]
    return np.array([[float(t.replace("D", "E")) for t in r] for r in rows])


def read_ener(path):
    """(time fs, T_el, T_ion, Epot+Um, Etot) rows of an ener*.dat file (result.f90:319-320)."""
    return _table(path)


def read_rdf(path):
    return _table(path)


def read_rest(path):
    """(x, v, f, ids) of a RESTnn.xyz file (result.f90:77-131)."""
    rows = pathlib.Path(path).read_text().splitlines()[2:]
    data = [r.split() for r in rows if r.strip()]
    a = np.array([[float(t) for t in r[1:10]] for r in data])
    ids = np.array([int(r[10]) for r in data])
    return a[:, 0:3], a[:, 3:6], a[:, 6:9], ids
