"""Build libtcpgpu.so (CUDA, sm_103a) in-tree with nvcc.

Every translation unit under csrc/ is compiled in parallel for
`-gencode arch=compute_103a,code=sm_103a` only, then linked into
tcp_allpair_gb300/_build/libtcpgpu.so against cuFFT and the shared CUDA
runtime.  Objects are rebuilt when their sources or headers are newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import pathlib
import shutil
import subprocess

PKG = pathlib.Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_build"
LIB = OUT / "libtcpgpu.so"
DRIVE = OUT / "tcp_drive"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-diag-suppress", "177",
              f"-I{ROOT / 'include'}", f"-I{CSRC}"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and pathlib.Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libtcpgpu.so")


def sources():
    return sorted(CSRC.glob("*.cu"))


def _stale(obj: pathlib.Path, src: pathlib.Path) -> bool:
    if not obj.exists():
        return True
    deps = [src] + list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    return any(d.stat().st_mtime > obj.stat().st_mtime for d in deps)


def build(verbose: bool = False, extra_flags=()) -> pathlib.Path:
    OUT.mkdir(exist_ok=True)
    cc = nvcc()
    jobs = []
    for src in sources():
        obj = OUT / (src.stem + ".o")
        if _stale(obj, src):
            jobs.append([cc, *ARCH, *NVCC_FLAGS, *extra_flags, "-c", str(src), "-o", str(obj)])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed ({' '.join(cmd)}):\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return r

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    objs = [str(OUT / (s.stem + ".o")) for s in sources()]
    if jobs or not LIB.exists():
        run([cc, *ARCH, "-shared", "-cudart", "shared", "-o", str(LIB), *objs, "-lcufft"])
    # host driver replaying main.f90 on the C ABI
    drive_src = CSRC / "host" / "tcp_drive.cpp"
    if not DRIVE.exists() or DRIVE.stat().st_mtime < max(drive_src.stat().st_mtime, LIB.stat().st_mtime):
        cxx = os.environ.get("CXX", "g++")
        run([cxx, "-O2", "-std=c++17", f"-I{ROOT / 'include'}", str(drive_src), "-o", str(DRIVE),
             f"-L{OUT}", "-ltcpgpu", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
