"""ctypes declarations of the C ABI in include/tcp_gpu.h.

This module only describes the boundary; it loads the in-tree
libtcpgpu.so and fails loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import pathlib

LIB_PATH = pathlib.Path(__file__).resolve().parent / "_build" / "libtcpgpu.so"

TCP_OK = 0
TCP_ERR_BAD_PARAM = 1
TCP_ERR_CUTOFF = 2
TCP_ERR_CUDA = 3
TCP_ERR_CUFFT = 4
TCP_ERR_TIMEOUT = 5
TCP_ERR_NO_DEVICE = 6
TCP_ERR_STATE = 7
TCP_ERR_NOMEM = 8

PREC_FP64, PREC_FP32C, PREC_FP32C_R64 = 0, 1, 2
EI_DEUTSCH, EI_KELBG, EI_COULOMB = 0, 1, 2
THERMO_NOTEMP, THERMO_ISOKIN, THERMO_BEREND, THERMO_STOCH = 0, 1, 2, 3
RECIP_NONE, RECIP_SPME, RECIP_EWALD = 0, 1, 2
FLAG_RDF, FLAG_VDF, FLAG_ENERGY, FLAG_DETERMINISTIC = 1, 2, 4, 8


class TcpParams(C.Structure):
    _fields_ = [
        ("xm", C.c_double * 2), ("q", C.c_double * 2), ("tau", C.c_double), ("alpha_lgv", C.c_double),
        ("a", C.c_double), ("box", C.c_double * 3), ("Te", C.c_double), ("Ti", C.c_double),
        ("rs", C.c_double), ("rc", C.c_double), ("K", C.c_int * 3), ("order", C.c_int),
        ("dx_ee", C.c_double), ("dx_ei", C.c_double), ("dx_ii", C.c_double),
        ("dv_e", C.c_double), ("dv_i", C.c_double), ("ei_model", C.c_int), ("lambda_ei", C.c_double),
        ("charge_scale", C.c_double), ("precision", C.c_int), ("reciprocal", C.c_int),
        ("ewald_nmax2", C.c_int), ("thermo", C.c_int), ("thermo_period", C.c_int), ("seed", C.c_uint64),
    ]


class TcpEnergies(C.Structure):
    _fields_ = [("Ur", C.c_double), ("Uo", C.c_double), ("Um", C.c_double), ("Epot", C.c_double),
                ("mv2el", C.c_double), ("mv2ion", C.c_double)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_P = C.POINTER(C.c_double)
_CTX = C.c_void_p

# name -> (restype, argtypes); the C declarations are in include/tcp_gpu.h
SIGNATURES = {
    "tcp_create": (C.c_int, [C.POINTER(TcpParams), C.c_int, C.c_int, C.c_int, C.POINTER(_CTX)]),
    "tcp_destroy": (C.c_int, [_CTX]),
    "tcp_last_error": (C.c_char_p, []),
    "tcp_status_string": (C.c_char_p, [C.c_int]),
    "tcp_version": (C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "tcp_ewald_self": (C.c_int, [_CTX, _P, _P]),
    "tcp_set_params": (C.c_int, [_CTX, C.POINTER(TcpParams)]),
    "tcp_set_flags": (C.c_int, [_CTX, C.c_uint]),
    "tcp_upload": (C.c_int, [_CTX, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_long]),
    "tcp_download": (C.c_int, [_CTX, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_long]),
    "tcp_upload_soa": (C.c_int, [_CTX, C.c_void_p, C.c_void_p, C.c_void_p]),
    "tcp_download_soa": (C.c_int, [_CTX, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "tcp_force_direct": (C.c_int, [_CTX, _P]),
    "tcp_force_direct_noalloc": (C.c_int, [C.POINTER(TcpParams), C.c_int, C.c_int, C.c_void_p, C.c_void_p, _P,
                                           C.c_void_p]),
    "tcp_force_spme": (C.c_int, [_CTX, _P]),
    "tcp_spme_sum": (C.c_int, [_CTX]),
    "tcp_remove_rigidmtn": (C.c_int, [_CTX]),
    "tcp_force": (C.c_int, [_CTX, C.POINTER(TcpEnergies)]),
    "tcp_vverlet1": (C.c_int, [_CTX, C.c_double]),
    "tcp_vverlet2": (C.c_int, [_CTX, C.c_double, _P, _P]),
    "tcp_finit": (C.c_int, [_CTX, C.c_double, C.POINTER(TcpEnergies)]),
    "tcp_md_steps": (C.c_int, [_CTX, C.c_double, C.c_int, C.POINTER(TcpEnergies)]),
    "tcp_md_steps_records": (C.c_int, [_CTX, C.c_double, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_long,
                                       C.c_void_p, C.c_void_p, C.c_void_p, C.c_long, C.POINTER(TcpEnergies)]),
    "tcp_energies_get": (C.c_int, [_CTX, C.POINTER(TcpEnergies)]),
    "tcp_histograms": (C.c_int, [_CTX, _P, _P, C.c_int]),
    "tcp_time_component": (C.c_int, [_CTX, C.c_int, C.c_int, C.c_double, _P]),
    "tcp_time_steps": (C.c_int, [_CTX, C.c_double, C.c_int, C.c_int, _P]),
    "tcp_autotune_report": (C.c_int, [_CTX, C.POINTER(C.c_int), _P, C.c_int]),
    "tcp_pair_variant_name": (C.c_char_p, [C.c_int]),
    "tcp_batch_variant_name": (C.c_char_p, [C.c_int]),
    "tcp_overlap_report": (C.c_int, [_CTX, C.POINTER(C.c_int), C.POINTER(C.c_int), _P, C.c_int]),
    "tcp_launch_count": (C.c_int, [_CTX, C.POINTER(C.c_longlong)]),
    "tcp_fp32_peak": (C.c_int, [C.c_int, _P]),
    "tcp_params_from_env": (C.c_int, [C.POINTER(TcpParams), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "tcp_adjoint_energy": (C.c_int, [_CTX, _P, _P, _P]),
    "tcp_hvp": (C.c_int, [_CTX, C.c_void_p, C.c_void_p, _P]),
    "tcp_reverse_md": (C.c_int, [_CTX, C.c_double, C.c_int, C.c_int, _P, _P]),
    "tcp_batch_create": (C.c_int, [C.POINTER(TcpParams), C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int, C.c_int,
                                   C.POINTER(C.c_void_p)]),
    "tcp_batch_destroy": (C.c_int, [C.c_void_p]),
    "tcp_batch_ewald_self": (C.c_int, [C.c_void_p, _P]),
    "tcp_batch_upload": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "tcp_batch_download": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    "tcp_batch_force": (C.c_int, [C.c_void_p, C.POINTER(TcpEnergies)]),
    "tcp_batch_md_steps": (C.c_int, [C.c_void_p, C.c_double, C.c_int, C.POINTER(TcpEnergies)]),
    "tcp_batch_time_steps": (C.c_int, [C.c_void_p, C.c_double, C.c_int, C.c_int, _P]),
    "tcp_batch_time_component": (C.c_int, [C.c_void_p, C.c_int, C.c_int, _P]),
    "tcp_batch_autotune_report": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), _P, C.c_int]),
    "tcp_batch_overlap_report": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), _P, C.c_int]),
}

_lib = None


def load(path: str | None = None):
    """Load libtcpgpu.so (built by tcp_allpair_gb300._build.build())."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = pathlib.Path(path) if path else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: run `python -c 'import __graft_entry__ as g; g.build()'` "
                           "(the CUDA library is required; there is no CPU fallback)")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class TcpError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where} failed with status {code}: {msg}")
        self.code = code


def check(lib, code: int, where: str):
    if code != TCP_OK:
        raise TcpError(code, where, (lib.tcp_last_error() or b"").decode())
