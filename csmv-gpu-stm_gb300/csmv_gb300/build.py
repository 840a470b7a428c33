"""In-tree build of the CSMV GB300 library and drivers (no cmake, no setup.py).

Compiles every CUDA/C++ translation unit of ``csrc/`` for sm_103a in parallel with nvcc, links
``lib/libcsmv.so`` (CUDA runtime linked statically, C ABI only), and the driver executables
``bin/csmv_bank`` / ``bin/csmv_memcd`` that keep the reference's command lines.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent  # csmv-gpu-stm_gb300/
REPO_ROOT = PKG_ROOT.parent
CSRC = PKG_ROOT / "csrc"
HOST = PKG_ROOT / "host"
BUILD = PKG_ROOT / "_build"
LIB = PKG_ROOT / "lib" / "libcsmv.so"
DEVTEST_LIB = PKG_ROOT / "lib" / "libcsmv_devtest.so"
BIN = PKG_ROOT / "bin"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-I", str(REPO_ROOT / "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CSMV library needs the CUDA 13 toolkit")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def build(verbose: bool = False) -> Path:
    """Build libcsmv.so and the drivers; returns the library path."""
    nv = nvcc()
    BUILD.mkdir(exist_ok=True)
    LIB.parent.mkdir(exist_ok=True)
    BIN.mkdir(exist_ok=True)
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(
        (REPO_ROOT / "include").glob("*"))
    units = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    jobs = []
    for src in units:
        obj = BUILD / (src.name + ".o")
        if _stale(obj, [src] + headers):
            jobs.append([nv, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for _ in ex.map(_run, jobs):
            pass
    objs = [BUILD / (s.name + ".o") for s in units]
    if _stale(LIB, objs):
        _run([nv, *ARCH, "-shared", "-o", str(LIB), *map(str, objs)])
    devtests = sorted((CSRC / "devtest").glob("*.cu"))
    if _stale(DEVTEST_LIB, devtests + headers):
        _run([nv, *ARCH, *NVCC_FLAGS, "-shared", *map(str, devtests), "-o", str(DEVTEST_LIB)])
    for main in sorted(HOST.glob("*.cpp")):
        exe = BIN / main.stem
        if _stale(exe, [main, LIB] + headers):
            _run([nv, "-O2", "-std=c++17", "-I", str(REPO_ROOT / "include"), str(main),
                  "-o", str(exe), "-L", str(LIB.parent), "-lcsmv",
                  "-Xlinker", "-rpath=$ORIGIN/../lib"])
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
