"""Build recipe for libzqs_gb300.so (hand-written sm_103a CUDA + C++ host).

Compiles every translation unit under csrc/ with nvcc in parallel into
_build/ and links lib/libzqs_gb300.so in-tree.  Numerics flags: no FMA
contraction (-fmad=false) and IEEE division / square root, so the FP32
kernels reproduce the CPU oracle's arithmetic exactly.
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
INCLUDE = PKG.parent / "include"
BUILD = PKG / "_build"
LIBDIR = PKG / "lib"
LIB = LIBDIR / "libzqs_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NUMERICS = ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]
# host code: no contraction either (the host-side arithmetic, e.g. image
# quantisation, must match the CPU restatement on x86 and Arm alike)
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-fvisibility=hidden,-O2,-ffp-contract=off",
          f"-I{INCLUDE}", f"-I{CSRC}"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libzqs_gb300.so")
    return exe


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    deps = [src] + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    t = obj.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: Path, extra: list[str]) -> Path:
    obj = BUILD / (src.name + ".o")
    if not _stale(obj, src):
        return obj
    cmd = [nvcc(), "-c", str(src), "-o", str(obj)] + ARCH + NUMERICS + COMMON + extra
    if src.suffix == ".cpp":
        cmd = [nvcc(), "-x", "cu", "-c", str(src), "-o", str(obj)] + ARCH + NUMERICS + COMMON + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Compile and link the library; returns the .so path."""
    extra = list(extra or [])
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    srcs = sources()
    if force:
        for s in srcs:
            o = BUILD / (s.name + ".o")
            if o.exists():
                o.unlink()
    workers = max(1, min(len(srcs), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(workers) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    if force or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), "-shared", "-o", str(tmp)] + ARCH + [str(o) for o in objs] + ["-cudart", "static"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


def ptxas_report(src_name: str) -> str:
    """-Xptxas -v register/spill report of one translation unit."""
    src = CSRC / src_name
    cmd = [nvcc(), "-c", str(src), "-o", os.devnull, "-Xptxas", "-v"] + ARCH + NUMERICS + COMMON
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.stdout + r.stderr


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    if "--ptxas" in sys.argv:
        for s in sources():
            if s.suffix == ".cu":
                print(ptxas_report(s.name))
