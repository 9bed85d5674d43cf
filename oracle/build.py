"""Build recipe for the CPU oracle (test infrastructure only).

Compiles ``oracle/*.c`` with gcc into ``oracle/_build/liboracle.so`` with
OpenMP and ``-ffp-contract=off`` (no fused multiply-add contraction, on x86
and on Arm alike), so its FP64 operation sequence matches the reference's
scalar code and the GPU's FP64 path.  The reference itself (Kokkos, Cabana,
MPI, n2p2) cannot be built in this environment, so there is no
``oracle/_ref``.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_build"


def build_oracle(verbose: bool = False) -> Path:
    OUT.mkdir(parents=True, exist_ok=True)
    lib = OUT / "liboracle.so"
    srcs = sorted(HERE.glob("*.c"))
    deps = srcs + sorted(HERE.glob("*.h"))
    if not lib.exists() or any(d.stat().st_mtime > lib.stat().st_mtime for d in deps):
        cc = os.environ.get("CC", "gcc")
        cmd = [cc, "-O2", "-std=c11", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
               "-fno-fast-math", "-Wall", "-o", str(lib)] + [str(s) for s in srcs] + ["-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {lib}")
    return lib


if __name__ == "__main__":
    build_oracle(verbose=True)
