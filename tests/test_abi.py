"""The C-ABI boundary (CPU only: no kernel is launched here).

libtcpgpu.so must load, export every entry point include/tcp_gpu.h
declares, agree with the ctypes declarations, and reject bad parameters
before touching a device.
"""
import ctypes as C
import pathlib
import re

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def lib():
    from tcp_allpair_gb300 import _abi, _build
    _build.build()
    return _abi.load()


def declared_functions():
    names = []
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        names += re.findall(r"^\s*(?:const\s+)?[a-z_]+\s*\*?\s*(tcp_[a-z0-9_]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "tcp_force_direct" in names and "tcp_md_steps" in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} declared in include/ but not exported"


def test_ctypes_declarations_cover_header():
    from tcp_allpair_gb300 import _abi
    assert set(declared_functions()) == set(_abi.SIGNATURES), "ctypes SIGNATURES out of sync with include/"


def test_struct_layout_matches_header():
    """tcp_params / tcp_energies sizes as the C compiler lays them out."""
    import subprocess
    import tempfile
    from tcp_allpair_gb300 import _abi
    src = ('#include <stdio.h>\n#include <stddef.h>\n#include "tcp_gpu.h"\n'
           'int main(void){printf("%zu %zu %zu %zu\\n", sizeof(tcp_params), sizeof(tcp_energies),'
           ' offsetof(tcp_params, seed), offsetof(tcp_params, lambda_ei)); return 0;}\n')
    with tempfile.TemporaryDirectory() as d:
        c = pathlib.Path(d) / "t.c"
        c.write_text(src)
        exe = pathlib.Path(d) / "t"
        subprocess.run(["gcc", "-I", str(ROOT / "include"), str(c), "-o", str(exe)], check=True)
        out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert int(out[0]) == C.sizeof(_abi.TcpParams)
    assert int(out[1]) == C.sizeof(_abi.TcpEnergies)
    assert int(out[2]) == _abi.TcpParams.seed.offset
    assert int(out[3]) == _abi.TcpParams.lambda_ei.offset


def test_bad_params_rejected_before_device(lib):
    from tcp_allpair_gb300 import _abi
    p = _abi.TcpParams()          # all zero: box <= 0
    h = C.c_void_p()
    code = lib.tcp_create(C.byref(p), 4, 4, 0, C.byref(h))
    assert code == _abi.TCP_ERR_BAD_PARAM
    assert b"box" in lib.tcp_last_error()
    assert lib.tcp_status_string(_abi.TCP_ERR_CUTOFF).startswith(b"cut-off")
    maj, mnr, arch = C.c_int(), C.c_int(), C.c_int()
    assert lib.tcp_version(C.byref(maj), C.byref(mnr), C.byref(arch)) == 0 and arch.value == 103


def test_pt_record_layout():
    """PT (data.f90:32-35): id + 12 doubles, 104-byte records."""
    from tcp_allpair_gb300.system import PT_DTYPE
    assert PT_DTYPE.itemsize == 104
    assert PT_DTYPE.fields["xx"][1] == 8 and PT_DTYPE.fields["xv"][1] == 32 and PT_DTYPE.fields["ff"][1] == 56
