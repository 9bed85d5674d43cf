"""Build recipe for libgbmd.so (the C-ABI CUDA library) and the host driver.

Compiles every ``csrc/*.cu`` for sm_103a only, in parallel, and links the
shared library in-tree at ``cabanamd_gb300/_lib/libgbmd.so``.  No CMake, no
torch extension machinery: the product is a plain C-ABI shared object.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
LIBDIR = PKG / "_lib"
OBJDIR = LIBDIR / "obj"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# CUDA 13 marks double4 deprecated (its 16-byte alignment is ambiguous next
# to the new double4_16a / double4_32a); the code relies on the 16-byte
# alignment of double4, so the notice is silenced rather than repeated for
# every use.
NVCC_FLAGS = [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-diag-suppress=1444",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2,-Wno-deprecated-declarations",
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgbmd")


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_lib(verbose: bool = False, extra_flags: list[str] | None = None) -> Path:
    """Compile csrc/*.cu -> _lib/libgbmd.so; returns the library path."""
    OBJDIR.mkdir(parents=True, exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    headers = sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    nv = nvcc()
    flags = ARCH + NVCC_FLAGS + ["-I", str(INCLUDE)] + (extra_flags or [])
    jobs = []
    objs = []
    for src in sources:
        obj = OBJDIR / (src.stem + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append([nv, "-c", str(src), "-o", str(obj)] + flags)
    if jobs:
        workers = min(len(jobs), os.cpu_count() or 4)
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            list(ex.map(_run, jobs))
    lib = LIBDIR / "libgbmd.so"
    if _stale(lib, objs):
        _run([nv, "-shared", "-o", str(lib)] + [str(o) for o in objs] + ARCH
             + ["-lcudart"])
    if verbose:
        print(f"built {lib}")
    return lib


def build_host(verbose: bool = False) -> Path | None:
    """Compile the C++ host driver (cbnmd_gb300) against libgbmd.so."""
    srcs = sorted(HOST.glob("*.cpp"))
    if not srcs:
        return None
    exe = LIBDIR / "cbnmd_gb300"
    deps = srcs + sorted(HOST.glob("*.h")) + sorted(INCLUDE.glob("*.h")) + [LIBDIR / "libgbmd.so"]
    if _stale(exe, deps):
        cxx = os.environ.get("CXX", "g++")
        _run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(INCLUDE), "-I", str(HOST)]
             + [str(s) for s in srcs]
             + ["-L", str(LIBDIR), "-lgbmd", f"-Wl,-rpath,{LIBDIR}", "-o", str(exe)])
    if verbose:
        print(f"built {exe}")
    return exe


if __name__ == "__main__":
    build_lib(verbose=True)
    build_host(verbose=True)
    sys.exit(0)
