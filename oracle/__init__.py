"""FP64 CPU oracle of the TCP_allpair force-and-integrate path.

TEST INFRASTRUCTURE ONLY.  This package is the checker the CUDA library is
compared against (tests/, __graft_entry__.smoke()) and the timed CPU
baseline of bench.py; the product never imports it.  The C restatement is in
tcp_oracle.c (citations to the reference inline) and is built by
oracle/Makefile into oracle/_build/liborc.so.

Parity status: unpinned by the reference (no reference tests or fixtures
exist and the Fortran/MPI/FFTE reference cannot be built on either machine);
pinned by analytic known answers in tests/test_oracle_*.py.
"""
from __future__ import annotations

import ctypes as C
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
LIB = HERE / "_build" / "liborc.so"
NDIST = 500
EPS = 14.399644154020082

EI = {"deutsch": 0, "kelbg": 1, "coulomb": 2}
THERMO = {"notemp": 0, "isokin": 1, "berend": 2, "stoch": 3}


class OrcParams(C.Structure):
    _fields_ = [
        ("xm", C.c_double * 2), ("q", C.c_double * 2), ("tau", C.c_double), ("alpha_lgv", C.c_double),
        ("a", C.c_double), ("box", C.c_double * 3), ("Te", C.c_double), ("Ti", C.c_double),
        ("rs", C.c_double), ("rc", C.c_double), ("rc2", C.c_double), ("K", C.c_int * 3), ("order", C.c_int),
        ("dx_ee", C.c_double), ("dx_ei", C.c_double), ("dx_ii", C.c_double), ("dv_e", C.c_double),
        ("dv_i", C.c_double), ("ei_model", C.c_int), ("lambda_ei", C.c_double), ("charge_scale", C.c_double),
    ]


def build():
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build()
        _lib = C.CDLL(str(LIB))
        D = C.POINTER(C.c_double)
        P = C.POINTER(OrcParams)
        sig = {
            "orc_ewald_self": (C.c_int, [P, C.c_int, C.c_int, C.c_double, D, D]),
            "orc_force_direct": (None, [P, C.c_int, C.c_int, D, D, D, D, C.c_int]),
            "orc_force_direct_rows": (None, [P, C.c_int, C.c_int, D, C.c_int, C.c_int, D, D, C.c_int]),
            "orc_force_spme": (C.c_int, [P, C.c_int, C.c_int, D, D, D, D]),
            "orc_bspline_moduli": (None, [C.c_int, C.c_int, D]),
            "orc_ewald_ksum": (None, [P, C.c_int, C.c_int, D, C.c_int, D, D, C.c_int]),
            "orc_spme_sum": (None, [C.c_int, D, D]),
            "orc_remove_rigidmtn": (None, [C.c_int, D]),
            "orc_vverlet1": (None, [P, C.c_int, C.c_int, C.c_double, D, D, D]),
            "orc_vverlet_stoch1": (None, [P, C.c_int, C.c_int, C.c_double, D, D, D]),
            "orc_vverlet2": (None, [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, D, D, D, D, D, D]),
            "orc_force_total": (C.c_int, [P, C.c_int, C.c_int, D, D, C.c_int, C.c_int, D, D, D, D, C.c_int]),
            "orc_finit": (C.c_int, [P, C.c_int, C.c_int, C.c_double, D, D, D, D, D, D, C.c_int]),
            "orc_md_step": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, D, D, D, D, C.c_double,
                                      C.c_int, C.c_int, D, D, D, C.c_int]),
            "orc_max_threads": (C.c_int, []),
            "orc_adjoint_energy": (None, [P, C.c_int, C.c_int, D, D, C.c_int]),
            "orc_hvp": (None, [P, C.c_int, C.c_int, D, D, C.c_int, C.c_int, D, D, D, C.c_int]),
            "orc_reverse_md": (C.c_int, [P, C.c_int, C.c_int, D, D, D, C.c_int, C.c_int, C.c_double, C.c_int,
                                         C.c_int, D, D, C.c_int]),
        }
        for k, (r, a) in sig.items():
            fn = getattr(_lib, k)
            fn.restype = r
            fn.argtypes = a
    return _lib


def _d(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    """FP64 restatement bound to one parameter set (reference units)."""

    def __init__(self, nel, nion, box, rc, xm=(1.0, 1836.0), q=(-1.0, 1.0), alpha=0.0, rs=1.0,
                 lambda_ei=1.0, ei="deutsch", K=0, order=4, Te=1.0, Ti=1.0, tau=1.0, alpha_lgv=0.0,
                 rdf_dx=None, charge_scale=1.0, nthreads=0):
        self.L = lib()
        self.nel, self.nion = nel, nion
        p = OrcParams()
        p.xm[0], p.xm[1] = xm
        p.q[0], p.q[1] = q
        p.tau, p.alpha_lgv = tau, alpha_lgv
        box = (box, box, box) if np.isscalar(box) else tuple(box)
        for d in range(3):
            p.box[d] = box[d]
            p.K[d] = K if np.isscalar(K) else K[d]
        p.Te, p.Ti, p.rs, p.rc = Te, Ti, rs, rc
        p.order = order
        dx = rdf_dx if rdf_dx is not None else rc / NDIST
        p.dx_ee = p.dx_ei = p.dx_ii = dx
        p.dv_e, p.dv_i = Te * 4.0 / NDIST, Ti * 4.0 / NDIST
        p.ei_model = EI[ei]
        p.lambda_ei = lambda_ei
        p.charge_scale = charge_scale
        self.p = p
        self.nthreads = nthreads
        kk = p.K[0] * p.K[1] * p.K[2]
        self.psi = np.zeros(max(kk, 1))
        uo = C.c_double()
        rc_ = self.L.orc_ewald_self(C.byref(p), nel, nion, alpha, _d(self.psi) if kk else None, C.byref(uo))
        if rc_ != 0:
            raise ValueError(" *** error at cut-off radius *** (rc > min(box)/2)")
        self.Uo = uo.value
        self.alpha = p.a

    @classmethod
    def from_system(cls, sys, ei="kelbg", **kw):
        args = dict(xm=sys.xm, q=sys.q, alpha=sys.alpha, rs=sys.lambda_ei, lambda_ei=sys.lambda_ei, ei=ei,
                    K=sys.K, order=sys.order, Te=sys.Te, Ti=sys.Ti)
        args.update(kw)
        return cls(sys.nel, sys.nion, sys.box, sys.rc, **args)

    @property
    def n(self):
        return self.nel + self.nion

    def force_direct(self, x, rdf=False):
        x = np.ascontiguousarray(x, dtype=np.float64)
        f = np.zeros((self.n, 3))
        ur = C.c_double()
        h = np.zeros(3 * (NDIST + 1)) if rdf else None
        self.L.orc_force_direct(C.byref(self.p), self.nel, self.nion, _d(x), _d(f), C.byref(ur), _d(h),
                                self.nthreads)
        return (f, ur.value, h.reshape(3, NDIST + 1)) if rdf else (f, ur.value)

    def force_direct_rows(self, x, i0, i1):
        x = np.ascontiguousarray(x, dtype=np.float64)
        f = np.zeros((i1 - i0, 3))
        ur = C.c_double()
        self.L.orc_force_direct_rows(C.byref(self.p), self.nel, self.nion, _d(x), i0, i1, _d(f), C.byref(ur),
                                     self.nthreads)
        return f, ur.value

    def force_spme(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        f = np.zeros((self.n, 3))
        um = C.c_double()
        self.L.orc_force_spme(C.byref(self.p), self.nel, self.nion, _d(x), _d(self.psi), _d(f), C.byref(um))
        return f, um.value

    def ewald_ksum(self, x, nmax2):
        x = np.ascontiguousarray(x, dtype=np.float64)
        f = np.zeros((self.n, 3))
        uk = C.c_double()
        self.L.orc_ewald_ksum(C.byref(self.p), self.nel, self.nion, _d(x), nmax2, _d(f), C.byref(uk),
                              self.nthreads)
        return f, uk.value

    def force_total(self, x, recip="spme", nmax2=64, rdf=False):
        x = np.ascontiguousarray(x, dtype=np.float64)
        f = np.zeros((self.n, 3))
        ur, um = C.c_double(), C.c_double()
        h = np.zeros(3 * (NDIST + 1)) if rdf else None
        r = {"none": 0, "spme": 1, "ewald": 2}[recip]
        self.L.orc_force_total(C.byref(self.p), self.nel, self.nion, _d(x), _d(self.psi), r, nmax2, _d(f),
                               C.byref(ur), C.byref(um), _d(h), self.nthreads)
        out = (f, ur.value, um.value)
        return out + (h.reshape(3, NDIST + 1),) if rdf else out

    def bspline_moduli(self, order, K):
        out = np.zeros(K)
        self.L.orc_bspline_moduli(order, K, _d(out))
        return out

    def vverlet1(self, x, v, f, dt, stoch=False):
        fn = self.L.orc_vverlet_stoch1 if stoch else self.L.orc_vverlet1
        fn(C.byref(self.p), self.nel, self.nion, dt, _d(x), _d(v), _d(f))

    def vverlet2(self, v, f, dt, thermo="notemp", apply=True, eta=None, vdf=False):
        a, b = C.c_double(), C.c_double()
        h = np.zeros(2 * (NDIST + 1)) if vdf else None
        self.L.orc_vverlet2(C.byref(self.p), THERMO[thermo], int(apply), self.nel, self.nion, dt, _d(v), _d(f),
                            _d(eta), C.byref(a), C.byref(b), _d(h))
        return (a.value, b.value, h.reshape(2, NDIST + 1)) if vdf else (a.value, b.value)

    def finit(self, x, v, dt):
        f = np.zeros((self.n, 3))
        ur, um = C.c_double(), C.c_double()
        self.L.orc_finit(C.byref(self.p), self.nel, self.nion, dt, _d(x), _d(v), _d(self.psi), _d(f),
                         C.byref(ur), C.byref(um), self.nthreads)
        return f, ur.value, um.value

    def md_step(self, x, v, f, dt, thermo="notemp", apply=True, recip="spme", nmax2=64):
        e = np.zeros(5)
        r = {"none": 0, "spme": 1, "ewald": 2}[recip]
        self.L.orc_md_step(C.byref(self.p), THERMO[thermo], int(apply), self.nel, self.nion, dt, _d(x), _d(v),
                           _d(f), _d(self.psi), self.Uo, r, nmax2, _d(e), None, None, self.nthreads)
        return dict(Ur=e[0], Um=e[1], Epot=e[2], mv2el=e[3], mv2ion=e[4])

    # ---- derivatives ----
    def dE_dlambda(self, x):
        """dE/dlambda_ei (Kelbg) or dE/drs (Deutsch) of the potential energy, eV/A."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        d = C.c_double()
        self.L.orc_adjoint_energy(C.byref(self.p), self.nel, self.nion, _d(x), C.byref(d), self.nthreads)
        return d.value

    def hvp(self, x, w, recip="spme", nmax2=64):
        """(H w, sum_i dF_i/dlambda . w_i), H the Hessian of the potential energy."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        w = np.ascontiguousarray(w, dtype=np.float64)
        hw = np.zeros((self.n, 3))
        d = C.c_double()
        r = {"none": 0, "spme": 1, "ewald": 2}[recip]
        self.L.orc_hvp(C.byref(self.p), self.nel, self.nion, _d(x), _d(self.psi), r, nmax2, _d(w), _d(hw),
                       C.byref(d), self.nthreads)
        return hw, d.value

    def reverse_md(self, x0, v0, dt, K, M, recip="spme", nmax2=64):
        """(J, dJ/dlambda): J = mean over K NOTEMP steps of (mv2el+mv2ion)/(3N)."""
        x0 = np.ascontiguousarray(x0, dtype=np.float64)
        v0 = np.ascontiguousarray(v0, dtype=np.float64)
        j, d = C.c_double(), C.c_double()
        r = {"none": 0, "spme": 1, "ewald": 2}[recip]
        self.L.orc_reverse_md(C.byref(self.p), self.nel, self.nion, _d(x0), _d(v0), _d(self.psi), r, nmax2, dt,
                              K, M, C.byref(j), C.byref(d), self.nthreads)
        return j.value, d.value

    def mean_temperature(self, x0, v0, dt, K, recip="spme", nmax2=64):
        """J of reverse_md by plain forward steps (for finite differences)."""
        x, v = x0.copy(), v0.copy()
        f, _, _ = self.force_total(x, recip=recip, nmax2=nmax2)
        acc = 0.0
        for _ in range(K):
            e = self.md_step(x, v, f, dt, recip=recip, nmax2=nmax2)
            acc += e["mv2el"] + e["mv2ion"]
        return acc / (3.0 * self.n * K)


def rms_rel(a, ref):
    """sqrt(sum |a - ref|^2 / sum |ref|^2) over particles."""
    a = np.asarray(a)
    ref = np.asarray(ref)
    return float(np.sqrt(np.sum((a - ref) ** 2) / np.sum(ref ** 2)))
