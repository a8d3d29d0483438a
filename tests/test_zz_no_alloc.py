"""tcp_force_direct_noalloc: the real-space sum for callers that cannot
allocate device memory (their HBM belongs to another allocator, or their step
loop forbids allocation after set-up because cudaMalloc/cudaFree can
synchronise the device).  It keeps its temporaries in a static 8 MiB device
array, so this test gives it device buffers that the test itself allocates
through the CUDA runtime and compares two calls in a row with the context
entry point tcp_force_direct.  Collected last on purpose.
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
    return rt


@pytest.mark.parametrize("precision,tol", [("fp32c", 1e-6), ("fp64", 1e-12)])
def test_noalloc_matches_context_entry_point(precision, tol):
    lib = _abi.load()
    rt = _cudart()
    s = T.make_system(3000, gamma=1.0, lam=0.5, seed=21, alpha_rc=3.1, K=16, order=4)
    p = T.params_for(s, precision=precision, ei="kelbg", recip="none")
    with T.Context(p, s.nel, s.nion) as c:          # the existing entry point
        c.EWALD_SELF()
        c.upload(x=s.x)
        ur_ref = c.Force_direct_self()
        _, _, f_ref, _ = c.download(x=False, v=False, f=True)

    n = s.n
    x_soa = np.ascontiguousarray(s.x.T)             # [3][n]
    nbytes = x_soa.nbytes
    dx, df = C.c_void_p(), C.c_void_p()
    assert rt.cudaMalloc(C.byref(dx), nbytes) == 0 and rt.cudaMalloc(C.byref(df), nbytes) == 0
    try:
        assert rt.cudaMemcpy(dx, x_soa.ctypes.data, nbytes, 1) == 0          # host -> device
        for call in range(2):                      # two calls in a row share the static scratch
            ur = C.c_double()
            rc = lib.tcp_force_direct_noalloc(C.byref(p), s.nel, s.nion, dx, df, C.byref(ur), None)
            assert rc == 0, lib.tcp_last_error()
            f_soa = np.empty((3, n))
            assert rt.cudaMemcpy(f_soa.ctypes.data, df, nbytes, 2) == 0      # device -> host
            f = f_soa.T
            assert oracle.rms_rel(f, f_ref) < tol, (call, oracle.rms_rel(f, f_ref))
            assert ur.value == pytest.approx(ur_ref, rel=tol)
    finally:
        rt.cudaFree(dx)
        rt.cudaFree(df)


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
