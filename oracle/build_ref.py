"""Build recipe for the reference's own CUDA kernels (TEST INFRASTRUCTURE ONLY).

Compiles four unmodified kernel files of the reference, where they lie in the
reference checkout, into device-only modules (cubins for sm_103a) under
oracle/_ref/:

    ZQ_SmokeSimulation3D/ZQ_CUDA_MACtoRegular.cu   -> mac.<flavour>.cubin
    ZQ_SmokeSimulation3D/ZQ_CUDA_Attenuation3D.cu  -> atten.<flavour>.cubin
    ZQ_SmokeSimulation3D/ZQ_CUDA_AddForce3D.cu     -> force.<flavour>.cubin
    ZQ_SmokeSimulation3D/ZQ_CUDA_Advection3D.cu    -> advect.<flavour>.cubin

Two flavours each:
  * "default": nvcc's default device flags, as the reference's Visual Studio
    project compiles them (ZQ_SmokeSimulation3D.vcxproj:102-104, 126-128 set
    no CUDA code-generation options), so FP32 multiply-adds may be contracted;
  * "nofma": -fmad=false, the arithmetic contract of the CPU oracle and of
    this library, so expression-for-expression agreement shows bit for bit.

Only headers of this directory are added: ref_shim/ZQlibCudaDefines.cuh and
ref_shim/ZQ_CUDA_PoissonSolver3D.cuh stand in for the un-vendored ZQlibCuda
headers the files include, and ref_shim/texref_shim.cuh (force-included for
the advection file) replaces the texture references that CUDA 12 removed.
No host code of the reference is compiled: oracle/ref_kernels.py loads the
modules through the CUDA driver API and restates the host wrappers' launch
sequences.

The modules are built where the reference checkout exists; elsewhere (a GPU
machine that only receives this repository) the prebuilt files in
oracle/_ref/ are used as they are.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SHIM = HERE / "ref_shim"
REF_DIR = Path(os.environ.get("ZQS_REFERENCE_DIR", "/root/reference")) / "ZQ_SmokeSimulation3D"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAVOURS = {"default": [], "nofma": ["-fmad=false"]}
MODULES = {
    "mac": ("ZQ_CUDA_MACtoRegular.cu", []),
    "atten": ("ZQ_CUDA_Attenuation3D.cu", []),
    "force": ("ZQ_CUDA_AddForce3D.cu", []),
    "advect": ("ZQ_CUDA_Advection3D.cu", ["-include", str(SHIM / "texref_shim.cuh")]),
}


def module_path(name: str, flavour: str) -> Path:
    return OUT / f"{name}.{flavour}.cubin"


def available() -> bool:
    return all(module_path(m, f).exists() for m in MODULES for f in FLAVOURS)


def _nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found")
    return exe


def _one(name: str, flavour: str, force: bool) -> Path:
    src_name, extra = MODULES[name]
    src = REF_DIR / src_name
    out = module_path(name, flavour)
    deps = [src, Path(__file__)] + list(SHIM.glob("*.cuh"))
    if not force and out.exists() and all(d.stat().st_mtime <= out.stat().st_mtime for d in deps):
        return out
    tmp = out.with_suffix(".tmp")
    cmd = [_nvcc(), "-cubin", "-o", str(tmp), str(src), f"-I{SHIM}", f"-I{REF_DIR}"] + ARCH + FLAVOURS[flavour] + extra
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference module build failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, out)
    return out


def build(force: bool = False) -> bool:
    """Builds the modules when the reference checkout is present; returns
    whether all modules exist afterwards."""
    if not REF_DIR.is_dir():
        return available()
    OUT.mkdir(exist_ok=True)
    jobs = [(m, f) for m in MODULES for f in FLAVOURS]
    with cf.ThreadPoolExecutor(min(len(jobs), os.cpu_count() or 4)) as ex:
        list(ex.map(lambda mf: _one(mf[0], mf[1], force), jobs))
    return available()


if __name__ == "__main__":
    print("reference modules:", "ok" if build(force="--force" in sys.argv) else "missing")
