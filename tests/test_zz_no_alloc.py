"""tcp_force_direct_noalloc: the real-space sum for callers that cannot
allocate device memory (their HBM belongs to another allocator, or their step
loop forbids allocation after set-up because cudaMalloc/cudaFree can
synchronise the device).  It keeps its temporaries in a static 8 MiB device
array, so this test gives it device buffers that the test itself allocates
through the CUDA runtime and compares two calls in a row with the context
entry point tcp_force_direct: both precisions, the three e-i models, a
non-cubic box with uneven species, and a stream the caller created.
Collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import oracle
import tcp_allpair_gb300 as T
from tcp_allpair_gb300 import _abi

pytestmark = pytest.mark.gpu

FP32_FORCE_RMS = 2e-6


def _cudart():
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            rt = C.CDLL(name)
            break
        except OSError:
            continue
    else:
        pytest.fail("libcudart not loadable")
    rt.cudaMalloc.argtypes = [C.POINTER(C.c_void_p), C.c_size_t]
    rt.cudaFree.argtypes = [C.c_void_p]
    rt.cudaMemcpy.argtypes = [C.c_void_p, C.c_void_p, C.c_size_t, C.c_int]
    rt.cudaDeviceSynchronize.argtypes = []
    rt.cudaStreamCreate.argtypes = [C.POINTER(C.c_void_p)]
    rt.cudaStreamDestroy.argtypes = [C.c_void_p]
    return rt


def _system(case, precision):
    """The test systems: a cubic box with each e-i model, and a box of
    (L, 1.1 L, 0.9 L) with uneven species (the general-box kernel path)."""
    s = T.make_system(3000, gamma=1.0, lam=0.5, seed=21, alpha_rc=3.1, K=16, order=4)
    ei = case.split("-")[1]
    box = None
    if case.startswith("noncubic"):
        rng = np.random.default_rng(5)
        s.nel, s.nion = 1700, 1300
        box = (s.box, 1.1 * s.box, 0.9 * s.box)
        s.x = (rng.random((s.n, 3)) - 0.5) * np.array(box)
    p = T.params_for(s, precision=precision, ei=ei, recip="none")
    if box is not None:
        for d in range(3):
            p.box[d] = box[d]
        p.rc = 0.45 * min(box)
        p.a = 3.1 / p.rc
    return s, p



def _context_forces(s, p, monkeypatch):
    # the context on its ordered-pair kernel, the one the no-alloc entry point
    # runs: its Newton-3 variants with the degree-5 erfc differ at the 1e-6 level
    monkeypatch.setenv("TCP_PAIR_VARIANT", "0")
    with T.Context(p, s.nel, s.nion) as c:          # the existing entry point
        c.EWALD_SELF()
        c.upload(x=s.x)
        ur = c.Force_direct_self()
        _, _, f, _ = c.download(x=False, v=False, f=True)
    return f, ur


def _noalloc_calls(lib, rt, s, p, stream, ncalls=2):
    n = s.n
    x_soa = np.ascontiguousarray(s.x.T)             # [3][n]
    nbytes = x_soa.nbytes
    dx, df = C.c_void_p(), C.c_void_p()
    assert rt.cudaMalloc(C.byref(dx), nbytes) == 0 and rt.cudaMalloc(C.byref(df), nbytes) == 0
    out = []
    try:
        assert rt.cudaMemcpy(dx, x_soa.ctypes.data, nbytes, 1) == 0          # host -> device
        for _ in range(ncalls):                    # calls in a row share the static scratch
            ur = C.c_double()
            rc = lib.tcp_force_direct_noalloc(C.byref(p), s.nel, s.nion, dx, df, C.byref(ur), stream)
            assert rc == 0, lib.tcp_last_error()
            f_soa = np.empty((3, n))
            assert rt.cudaMemcpy(f_soa.ctypes.data, df, nbytes, 2) == 0      # device -> host
            out.append((f_soa.T.copy(), ur.value))
    finally:
        rt.cudaFree(dx)
        rt.cudaFree(df)
    return out


@pytest.mark.parametrize("case", ["cubic-kelbg", "cubic-coulomb", "cubic-deutsch", "noncubic-kelbg"])
@pytest.mark.parametrize("precision,tol", [("fp32c", 1e-6), ("fp64", 1e-12)])
def test_noalloc_matches_context_entry_point(precision, tol, case, monkeypatch):
    lib = _abi.load()
    rt = _cudart()
    s, p = _system(case, precision)
    f_ref, ur_ref = _context_forces(s, p, monkeypatch)
    for call, (f, ur) in enumerate(_noalloc_calls(lib, rt, s, p, None)):
        assert oracle.rms_rel(f, f_ref) < tol, (call, oracle.rms_rel(f, f_ref))
        assert ur == pytest.approx(ur_ref, rel=tol)


def test_noalloc_on_a_created_stream(monkeypatch):
    """The caller's own stream instead of the legacy default stream."""
    lib = _abi.load()
    rt = _cudart()
    s, p = _system("cubic-kelbg", "fp32c")
    f_ref, ur_ref = _context_forces(s, p, monkeypatch)
    st = C.c_void_p()
    assert rt.cudaStreamCreate(C.byref(st)) == 0
    try:
        for f, ur in _noalloc_calls(lib, rt, s, p, st):
            assert oracle.rms_rel(f, f_ref) < 1e-6
            assert ur == pytest.approx(ur_ref, rel=1e-6)
    finally:
        rt.cudaStreamDestroy(st)


def test_noalloc_rejects_oversize():
    lib = _abi.load()
    s = T.make_system(64, seed=1, alpha_rc=3.1)
    p = T.params_for(s, precision="fp32c", ei="kelbg", recip="none")
    ur = C.c_double()
    big = 400_000
    rc = lib.tcp_force_direct_noalloc(C.byref(p), big // 2, big // 2, C.c_void_p(1), C.c_void_p(1),
                                      C.byref(ur), None)
    assert rc == _abi.TCP_ERR_BAD_PARAM
    assert b"8 MiB" in lib.tcp_last_error()
