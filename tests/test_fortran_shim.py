"""The Fortran drop-in boundary (CPU only: no Fortran compiler exists here).

tcp_allpair_gb300/fortran/tcp_gpu_mod.f90 replaces force.f90 and vverlet.f90
in the reference's build.  Every routine that main.f90 and init.f90 call in
those two files must exist in the module with the reference's dummy
arguments, or the unchanged main.f90 would not link.  The reference's
interface is recorded in tests/golden/reference_calls.json (written from the
reference's sources by tests/golden/make_reference_calls.py); when the
sources are present the fixture is checked against them too.

tcp_params_from_env() supplies the GPU build's own parameters (precision,
e-i model, order, alpha, lambda, device) that tcp.prm has no field for.
"""
import ctypes as C
import importlib.util
import json
import pathlib

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
SHIM = ROOT / "tcp_allpair_gb300" / "fortran" / "tcp_gpu_mod.f90"
FIXTURE = ROOT / "tests" / "golden" / "reference_calls.json"
REFERENCE = pathlib.Path("/root/reference")


def _gen():
    spec = importlib.util.spec_from_file_location("make_reference_calls",
                                                  ROOT / "tests" / "golden" / "make_reference_calls.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_shim_defines_every_routine_the_reference_calls():
    gen = _gen()
    ref = json.loads(FIXTURE.read_text())
    shim = gen.definitions(SHIM)
    called = sorted({c["name"] for c in ref["calls"]})
    assert len(called) == 13
    for name in called:
        assert name in shim, f"{name} is called at " + ", ".join(
            f"{c['file']}:{c['line']}" for c in ref["calls"] if c["name"] == name) + " but not defined by the module"
        want = [a.lower() for a in ref["definitions"][name]["args"]]
        got = [a.lower() for a in shim[name]["args"]]
        assert got == want, f"{name}: module has ({', '.join(got)}), reference ({', '.join(want)})"


def test_call_sites_pass_the_defined_arguments():
    """Each call passes the definition's arguments; init.f90 passes an extra
    PRE_data to Force_direct_self and Force_direct_ext (init.f90:195, 202,
    215), which implicit interfaces tolerate, as the reference relies on."""
    ref = json.loads(FIXTURE.read_text())
    extra = []
    for c in ref["calls"]:
        n = len(ref["definitions"][c["name"]]["args"])
        assert c["nargs"] >= n, c
        if c["nargs"] > n:
            extra.append((c["file"], c["name"]))
    assert all(f == "init.f90" for f, _ in extra)
    assert {n for _, n in extra} == {"FORCE_DIRECT_SELF", "FORCE_DIRECT_EXT"}


def test_module_routines_after_the_module_are_reference_names(tmp_path):
    """The drop-in routines (outside MODULE TCP_GPU) are exactly the called
    reference routines: nothing else that could clash with main.f90,
    init.f90 or result.f90 at link time."""
    gen = _gen()
    text = SHIM.read_text()
    tail = tmp_path / "tail.f90"
    tail.write_text(text[text.index("END MODULE TCP_GPU"):])
    outside = set(gen.definitions(tail))
    ref = json.loads(FIXTURE.read_text())
    assert outside == {c["name"] for c in ref["calls"]}


@pytest.mark.skipif(not (REFERENCE / "main.f90").exists(), reason="reference sources not present")
def test_fixture_matches_reference_sources():
    gen = _gen()
    assert gen.extract(REFERENCE) == json.loads(FIXTURE.read_text())


# ---- tcp_params_from_env -----------------------------------------------------
@pytest.fixture(scope="module")
def lib():
    from tcp_allpair_gb300 import _abi, _build
    _build.build()
    return _abi.load()


def _params():
    from tcp_allpair_gb300 import TcpParams
    p = TcpParams()
    p.order, p.precision, p.ei_model, p.lambda_ei, p.reciprocal = 4, 0, 0, 1.0, 1
    return p


def test_knobs_from_file_and_environment(lib, tmp_path, monkeypatch):
    for k in ("PRECISION", "EI_MODEL", "ORDER", "ALPHA", "LAMBDA_EI", "DEVICE", "SYNC_EVERY", "RECIPROCAL"):
        monkeypatch.delenv(f"TCP_GPU_{k}", raising=False)
    prm = tmp_path / "tcp_gpu.prm"
    prm.write_text("# GPU build parameters\nprecision = fp32c\nei_model kelbg   ! Kelbg e-i\norder 5\n"
                   "alpha = 1.25D-1\nlambda_ei 7.2\ndevice 0\nsync_every 10\n")
    monkeypatch.setenv("TCP_GPU_PRM", str(prm))
    monkeypatch.setenv("TCP_GPU_ORDER", "6")               # the environment wins over the file
    p, dev, sync = _params(), C.c_int(3), C.c_int(1)
    assert lib.tcp_params_from_env(C.byref(p), C.byref(dev), C.byref(sync)) == 0, lib.tcp_last_error()
    assert (p.precision, p.ei_model, p.order, p.reciprocal) == (1, 1, 6, 1)
    assert p.a == pytest.approx(0.125) and p.lambda_ei == pytest.approx(7.2)
    assert (dev.value, sync.value) == (0, 10)


def test_knobs_defaults_and_errors(lib, tmp_path, monkeypatch):
    from tcp_allpair_gb300 import _abi
    monkeypatch.chdir(tmp_path)                             # no ./tcp_gpu.prm
    monkeypatch.delenv("TCP_GPU_PRM", raising=False)
    for k in ("PRECISION", "EI_MODEL", "ORDER", "ALPHA", "LAMBDA_EI", "DEVICE", "SYNC_EVERY"):
        monkeypatch.delenv(f"TCP_GPU_{k}", raising=False)
    p = _params()
    assert lib.tcp_params_from_env(C.byref(p), None, None) == 0
    assert (p.precision, p.order) == (0, 4)                 # untouched without keys
    monkeypatch.setenv("TCP_GPU_PRECISION", "fp32c_r64")
    assert lib.tcp_params_from_env(C.byref(p), None, None) == 0 and p.precision == 2
    monkeypatch.setenv("TCP_GPU_ORDER", "9")
    assert lib.tcp_params_from_env(C.byref(p), None, None) == _abi.TCP_ERR_BAD_PARAM
    assert b"TCP_GPU_ORDER" in lib.tcp_last_error()
    monkeypatch.delenv("TCP_GPU_ORDER")
    (tmp_path / "tcp_gpu.prm").write_text("precision fp32c\nwarp_speed 9\n")
    assert lib.tcp_params_from_env(C.byref(p), None, None) == _abi.TCP_ERR_BAD_PARAM
    assert b"tcp_gpu.prm:2" in lib.tcp_last_error() and b"warp_speed" in lib.tcp_last_error()
    monkeypatch.setenv("TCP_GPU_PRM", str(tmp_path / "missing.prm"))
    assert lib.tcp_params_from_env(C.byref(p), None, None) == _abi.TCP_ERR_BAD_PARAM
