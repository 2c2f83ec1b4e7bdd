"""Build recipe of the CPU oracle (test infrastructure only).

g++ -O3 -fopenmp -ffp-contract=off: no contraction so FP32 arithmetic is
exactly the sequence written in zqs_oracle.cpp, which the CUDA kernels
reproduce.  Output: oracle/_build/libzqs_oracle.so (git-ignored).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
SRC = HERE / "zqs_oracle.cpp"
OUT = HERE / "_build" / "libzqs_oracle.so"
FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
         "-fvisibility=hidden"]


def build(force: bool = False) -> Path:
    OUT.parent.mkdir(exist_ok=True)
    deps = [SRC, HERE.parent / "include" / "zqs_capi.h", Path(__file__)]
    if not force and OUT.exists() and all(d.stat().st_mtime <= OUT.stat().st_mtime for d in deps):
        return OUT
    cxx = shutil.which("g++") or "g++"
    tmp = OUT.with_suffix(".so.tmp")
    cmd = [cxx] + FLAGS + [str(SRC), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
