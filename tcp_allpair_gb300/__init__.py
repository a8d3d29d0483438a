"""GB300-native force-and-integrate step of the TCP_allpair two-component
plasma code, behind the C ABI of libtcpgpu.so (include/tcp_gpu.h).

`Context` mirrors the reference's step routines one to one (force.f90,
vverlet.f90, init.f90): the method names are the Fortran subroutine names,
the arrays are the PT records of data.f90:32-35 (numpy structured arrays,
`system.PT_DTYPE`) and errors raise `TcpError` where the reference STOPs.
Compute always runs in libtcpgpu.so on the GPU; importing this package
without the built library, or calling it without a GB300, raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _abi
from ._abi import (EI_COULOMB, EI_DEUTSCH, EI_KELBG, FLAG_DETERMINISTIC, FLAG_ENERGY, FLAG_RDF, FLAG_VDF, PREC_FP32C,
                   PREC_FP32C_R64,
                   PREC_FP64, RECIP_EWALD, RECIP_NONE, RECIP_SPME, THERMO_BEREND, THERMO_ISOKIN,
                   THERMO_NOTEMP, THERMO_STOCH, TcpEnergies, TcpError, TcpParams)
from .system import EPS, NDIST, PT_DTYPE, System, make_config_system, make_system

__all__ = ["Context", "Batch", "TcpParams", "TcpEnergies", "TcpError", "params_for", "System", "make_system",
           "make_config_system", "PT_DTYPE", "EPS", "NDIST"]

_THERMO = {"notemp": THERMO_NOTEMP, "isokin": THERMO_ISOKIN, "berend": THERMO_BEREND, "stoch": THERMO_STOCH}
_EI = {"deutsch": EI_DEUTSCH, "kelbg": EI_KELBG, "coulomb": EI_COULOMB}
_RECIP = {"none": RECIP_NONE, "spme": RECIP_SPME, "ewald": RECIP_EWALD}
_PREC = {"fp64": PREC_FP64, "fp32c": PREC_FP32C, "fp32c_r64": PREC_FP32C_R64}


def params_for(sys: System, precision="fp32c", ei="kelbg", recip="spme", thermo="notemp",
               thermo_period=1, nmax2=64, tau=1.0, alpha_lgv=0.0, seed=0, charge_scale=1.0,
               rdf_dx=None) -> TcpParams:
    """TcpParams for a generated system (reference units)."""
    p = TcpParams()
    p.xm[0], p.xm[1] = sys.xm
    p.q[0], p.q[1] = sys.q
    p.tau, p.alpha_lgv = tau, alpha_lgv
    p.a = sys.alpha
    for d in range(3):
        p.box[d] = sys.box
        p.K[d] = sys.K
    p.Te, p.Ti = sys.Te, sys.Ti
    p.rs = sys.lambda_ei
    p.rc = sys.rc
    p.order = sys.order
    dx = rdf_dx if rdf_dx is not None else sys.rc / NDIST
    p.dx_ee = p.dx_ei = p.dx_ii = dx
    p.dv_e = sys.Te * 4.0 / NDIST          # main.f90:286-287
    p.dv_i = sys.Ti * 4.0 / NDIST
    p.ei_model = _EI[ei]
    p.lambda_ei = sys.lambda_ei
    p.charge_scale = charge_scale
    p.precision = _PREC[precision]
    p.reciprocal = _RECIP[recip]
    p.ewald_nmax2 = nmax2
    p.thermo = _THERMO[thermo]
    p.thermo_period = thermo_period
    p.seed = seed
    return p


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Context:
    """One system resident on one GB300 (a tcp_ctx of the C ABI)."""

    def __init__(self, params: TcpParams, nel: int, nion: int, device: int = 0):
        self.lib = _abi.load()
        self.params = params
        self.nel, self.nion = nel, nion
        h = C.c_void_p()
        _abi.check(self.lib, self.lib.tcp_create(C.byref(params), nel, nion, device, C.byref(h)), "tcp_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.tcp_destroy(self.h)
            self.h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _chk(self, code, where):
        _abi.check(self.lib, code, where)

    @property
    def n(self):
        return self.nel + self.nion

    # ---- reference routine names --------------------------------------------
    def EWALD_SELF(self):
        """force.f90:4-49 -> (alpha, Uo without eps)."""
        a, uo = C.c_double(), C.c_double()
        self._chk(self.lib.tcp_ewald_self(self.h, C.byref(a), C.byref(uo)), "tcp_ewald_self")
        return a.value, uo.value

    def Force_direct_self(self):
        """force.f90:52-372 over the whole system -> Ur (no eps); f overwritten."""
        u = C.c_double()
        self._chk(self.lib.tcp_force_direct(self.h, C.byref(u)), "tcp_force_direct")
        return u.value

    def Force_SPME4(self):
        """force.f90:652-929 -> Um (with eps); reciprocal forces stay on the device."""
        u = C.c_double()
        self._chk(self.lib.tcp_force_spme(self.h, C.byref(u)), "tcp_force_spme")
        return u.value

    def SPME_SUM(self):
        self._chk(self.lib.tcp_spme_sum(self.h), "tcp_spme_sum")

    def REMOVE_RIGIDMTN(self):
        self._chk(self.lib.tcp_remove_rigidmtn(self.h), "tcp_remove_rigidmtn")

    def VVerlet1(self, dt):
        """VVerletNotemp1 / VVerletStoch1 (vverlet.f90:132-171 / 9-59)."""
        self._chk(self.lib.tcp_vverlet1(self.h, dt), "tcp_vverlet1")

    def VVerlet2(self, dt):
        """VVerletNotemp2 / Isokin2 / Berend2 / Stoch2 -> (mv2el, mv2ion)."""
        a, b = C.c_double(), C.c_double()
        self._chk(self.lib.tcp_vverlet2(self.h, dt, C.byref(a), C.byref(b)), "tcp_vverlet2")
        return a.value, b.value

    def Finit(self, dt):
        e = TcpEnergies()
        self._chk(self.lib.tcp_finit(self.h, dt, C.byref(e)), "tcp_finit")
        return e.as_dict()

    # ---- composite -------------------------------------------------------------
    def force(self):
        e = TcpEnergies()
        self._chk(self.lib.tcp_force(self.h, C.byref(e)), "tcp_force")
        return e.as_dict()

    def md_steps(self, dt, nsteps):
        e = TcpEnergies()
        self._chk(self.lib.tcp_md_steps(self.h, dt, nsteps, C.byref(e)), "tcp_md_steps")
        return e.as_dict()

    def md_steps_pt(self, dt, nsteps, qel: np.ndarray, qion: np.ndarray, fields=("xx", "xv", "ff")):
        """nsteps steps on PT records (data.f90:32-35) updated in place, as
        main.f90:81-153 updates qel / qion: upload_pt + md_steps + download_pt
        in one call with one wait for the device."""
        ptr = []
        for arr in (qel, qion):
            offs = {k: arr.dtype.fields[k][1] for k in ("xx", "xv", "ff")}
            base = arr.ctypes.data
            live = len(arr) > 0
            ptr += [C.c_void_p(base + offs[k]) if (live and k in fields) else None for k in ("xx", "xv", "ff")]
            ptr.append(arr.strides[0] if live else 24)
        e = TcpEnergies()
        self._chk(self.lib.tcp_md_steps_records(self.h, dt, nsteps, *ptr, C.byref(e)), "tcp_md_steps_records")
        return e.as_dict()

    def set_flags(self, flags):
        self._chk(self.lib.tcp_set_flags(self.h, flags), "tcp_set_flags")

    def set_params(self, params: TcpParams):
        self._chk(self.lib.tcp_set_params(self.h, C.byref(params)), "tcp_set_params")
        self.params = params

    # ---- transfers ---------------------------------------------------------------
    def upload_pt(self, qel: np.ndarray, qion: np.ndarray, fields=("xx", "xv", "ff")):
        """Copy PT records (data.f90:32-35) to the device."""
        for sp, arr in ((0, qel), (1, qion)):
            if len(arr) == 0:
                continue
            base = arr.ctypes.data
            offs = {k: arr.dtype.fields[k][1] for k in ("xx", "xv", "ff")}
            ptr = [C.c_void_p(base + offs[k]) if k in fields else None for k in ("xx", "xv", "ff")]
            self._chk(self.lib.tcp_upload(self.h, sp, *ptr, arr.strides[0]), "tcp_upload")

    def download_pt(self, qel: np.ndarray, qion: np.ndarray, fields=("xx", "xv", "ff")):
        for sp, arr in ((0, qel), (1, qion)):
            if len(arr) == 0:
                continue
            base = arr.ctypes.data
            offs = {k: arr.dtype.fields[k][1] for k in ("xx", "xv", "ff")}
            ptr = [C.c_void_p(base + offs[k]) if k in fields else None for k in ("xx", "xv", "ff")]
            self._chk(self.lib.tcp_download(self.h, sp, *ptr, arr.strides[0]), "tcp_download")

    def upload(self, x=None, v=None, f=None):
        """(N,3) float64 arrays, electrons first."""
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (x, v, f)]
        for a in arrs:
            if a is not None and a.shape != (self.n, 3):
                raise ValueError(f"expected shape ({self.n}, 3), got {a.shape}")
        self._chk(self.lib.tcp_upload_soa(self.h, *[None if a is None else _ptr(a) for a in arrs]),
                  "tcp_upload_soa")

    def download(self, x=True, v=True, f=True, frec=False):
        out = [np.empty((self.n, 3)) if w else None for w in (x, v, f, frec)]
        self._chk(self.lib.tcp_download_soa(self.h, *[None if a is None else _ptr(a) for a in out]),
                  "tcp_download_soa")
        return out

    def histograms(self, reset=False):
        rdf = np.zeros(3 * (NDIST + 1))
        vdf = np.zeros(2 * (NDIST + 1))
        self._chk(self.lib.tcp_histograms(self.h, rdf.ctypes.data_as(C.POINTER(C.c_double)),
                                          vdf.ctypes.data_as(C.POINTER(C.c_double)), int(reset)),
                  "tcp_histograms")
        return rdf.reshape(3, NDIST + 1), vdf.reshape(2, NDIST + 1)

    def time_component(self, which, reps, dt=0.0):
        ms = C.c_double()
        self._chk(self.lib.tcp_time_component(self.h, which, reps, dt, C.byref(ms)), "tcp_time_component")
        return ms.value

    def time_steps(self, dt, nsteps, flush_l2=True):
        """Per-step CUDA-event timing: dict of summed ms per phase."""
        out = np.zeros(6)
        self._chk(self.lib.tcp_time_steps(self.h, dt, nsteps, int(flush_l2),
                                          out.ctypes.data_as(C.POINTER(C.c_double))), "tcp_time_steps")
        keys = ("step", "vverlet1", "recip", "pair", "epilogue", "nsteps")
        return dict(zip(keys, out.tolist()))

    def autotune_report(self):
        """(chosen FP32C pair-kernel variant, per-variant ms measured by the autotuner)."""
        v = C.c_int()
        ms = np.zeros(32)
        self._chk(self.lib.tcp_autotune_report(self.h, C.byref(v), ms.ctypes.data_as(C.POINTER(C.c_double)), 32),
                  "tcp_autotune_report")
        return v.value, ms

    def variant_name(self, variant):
        """Name of FP32C real-space variant `variant` (tcp_pair_variant_name)."""
        n = self.lib.tcp_pair_variant_name(int(variant))
        return n.decode() if n else None

    def overlap_report(self):
        """(CTAs left out of the Newton-3 grid, {candidate: ms of the pair kernel with the
        reciprocal chain beside it})."""
        r = C.c_int()
        cand = np.zeros(8, dtype=np.int32)
        ms = np.zeros(8)
        self._chk(self.lib.tcp_overlap_report(self.h, C.byref(r), cand.ctypes.data_as(C.POINTER(C.c_int)),
                                              ms.ctypes.data_as(C.POINTER(C.c_double)), 8), "tcp_overlap_report")
        return r.value, {int(k): float(t) for k, t in zip(cand, ms) if t > 0}

    def launch_count(self):
        n = C.c_longlong()
        self._chk(self.lib.tcp_launch_count(self.h, C.byref(n)), "tcp_launch_count")
        return n.value

    # ---- derivatives (tcp_adjoint_energy / tcp_hvp / tcp_reverse_md) ----
    def adjoint_energy(self):
        """(E, dE/dlambda, dE/ds) at the current positions (eV, eV/A, eV)."""
        e, dl, ds = C.c_double(), C.c_double(), C.c_double()
        self._chk(self.lib.tcp_adjoint_energy(self.h, C.byref(e), C.byref(dl), C.byref(ds)), "tcp_adjoint_energy")
        return e.value, dl.value, ds.value

    def hvp(self, w):
        """(H w, dF/dlambda . w) for w of shape (N, 3)."""
        w = np.ascontiguousarray(w, dtype=np.float64)
        hw = np.zeros_like(w)
        d = C.c_double()
        self._chk(self.lib.tcp_hvp(self.h, w.ctypes.data, hw.ctypes.data, C.byref(d)), "tcp_hvp")
        return hw, d.value

    def reverse_md(self, dt, nsteps, every):
        """(J, dJ/dlambda): J = mean over nsteps NOTEMP steps of (mv2el+mv2ion)/(3N)."""
        j, d = C.c_double(), C.c_double()
        self._chk(self.lib.tcp_reverse_md(self.h, dt, nsteps, every, C.byref(j), C.byref(d)), "tcp_reverse_md")
        return j.value, d.value


class Batch:
    """Many independent systems stepped together (tcp_batch_* of the C ABI)."""

    def __init__(self, params: list, nel: list, nion: list, device: int = 0):
        self.lib = _abi.load()
        self.nrep = len(params)
        self._params = (TcpParams * self.nrep)(*params)
        self._nel = (C.c_int * self.nrep)(*nel)
        self._nion = (C.c_int * self.nrep)(*nion)
        self.n = [a + b for a, b in zip(nel, nion)]
        h = C.c_void_p()
        _abi.check(self.lib, self.lib.tcp_batch_create(self._params, self._nel, self._nion, self.nrep, device,
                                                       C.byref(h)), "tcp_batch_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.tcp_batch_destroy(self.h)
            self.h = None

    __del__ = close

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _chk(self, code, where):
        _abi.check(self.lib, code, where)

    def EWALD_SELF(self):
        uo = np.zeros(self.nrep)
        self._chk(self.lib.tcp_batch_ewald_self(self.h, uo.ctypes.data_as(C.POINTER(C.c_double))),
                  "tcp_batch_ewald_self")
        return uo

    def upload(self, rep, x=None, v=None, f=None):
        arrs = [None if a is None else np.ascontiguousarray(a, dtype=np.float64) for a in (x, v, f)]
        self._chk(self.lib.tcp_batch_upload(self.h, rep, *[None if a is None else _ptr(a) for a in arrs]),
                  "tcp_batch_upload")

    def download(self, rep, x=True, v=True, f=True):
        out = [np.empty((self.n[rep], 3)) if w else None for w in (x, v, f)]
        self._chk(self.lib.tcp_batch_download(self.h, rep, *[None if a is None else _ptr(a) for a in out]),
                  "tcp_batch_download")
        return out

    def _energies(self, call, *args):
        e = (TcpEnergies * self.nrep)()
        self._chk(call(self.h, *args, e), call.__name__)
        return [x.as_dict() for x in e]

    def force(self):
        return self._energies(self.lib.tcp_batch_force)

    def md_steps(self, dt, nsteps):
        return self._energies(self.lib.tcp_batch_md_steps, C.c_double(dt), C.c_int(nsteps))

    def time_steps(self, dt, nsteps, flush_l2=True):
        """Per-step CUDA-event timing of the batched step: dict of summed ms per phase
        (the SPME chains run beside the pair launch)."""
        out = np.zeros(6)
        self._chk(self.lib.tcp_batch_time_steps(self.h, dt, nsteps, int(flush_l2),
                                                out.ctypes.data_as(C.POINTER(C.c_double))), "tcp_batch_time_steps")
        keys = ("step", "vverlet1", "recip", "pair", "epilogue", "nsteps")
        return dict(zip(keys, out.tolist()))

    def time_component(self, which, reps):
        """Mean ms of one launch of the batched pair kernel alone (which=0) or of the
        SPME chains of every replica alone (which=1), tcp_batch_time_component."""
        ms = C.c_double()
        self._chk(self.lib.tcp_batch_time_component(self.h, int(which), int(reps), C.byref(ms)),
                  "tcp_batch_time_component")
        return ms.value

    def autotune_report(self):
        """(chosen batched pair-kernel variant, per-variant ms measured by the batch autotuner)."""
        v = C.c_int()
        ms = np.zeros(16)
        self._chk(self.lib.tcp_batch_autotune_report(self.h, C.byref(v), ms.ctypes.data_as(C.POINTER(C.c_double)), 16),
                  "tcp_batch_autotune_report")
        return v.value, ms

    def variant_name(self, variant):
        """Name of batched real-space variant `variant` (tcp_batch_variant_name)."""
        n = self.lib.tcp_batch_variant_name(int(variant))
        return n.decode() if n else None

    def overlap_report(self):
        """(CTAs left out of the batched pair grid for the SPME chains, {candidate: ms of the
        pair launch with the chains beside it})."""
        r = C.c_int()
        cand = np.zeros(8, dtype=np.int32)
        ms = np.zeros(8)
        self._chk(self.lib.tcp_batch_overlap_report(self.h, C.byref(r), cand.ctypes.data_as(C.POINTER(C.c_int)),
                                                    ms.ctypes.data_as(C.POINTER(C.c_double)), 8),
                  "tcp_batch_overlap_report")
        return r.value, {int(k): float(t) for k, t in zip(cand, ms) if t > 0}


def fp32_peak(device: int = 0) -> float:
    """Measured FP32 FFMA rate of the device in 1e12 FFMA/s."""
    lib = _abi.load()
    t = C.c_double()
    _abi.check(lib, lib.tcp_fp32_peak(device, C.byref(t)), "tcp_fp32_peak")
    return t.value
