"""C ABI checks that need no GPU: the library builds, loads and exports every
entry point include/*.h declares; the headers compile as C and C++; the
parameter struct layout matches the C definition."""
import ctypes as C
import re
import shutil
import subprocess
from pathlib import Path

import pytest

from zq_smokesimulation_gb300 import capi

ROOT = Path(__file__).resolve().parents[1]
INC = ROOT / "include"


def declared_c_symbols():
    names = set()
    for h in INC.glob("*.h"):
        text = h.read_text()
        for m in re.finditer(r"ZQS_API\s+[\w\s\*]+?\b(\w+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_library_exports_every_declared_symbol(zqs_lib):
    declared = declared_c_symbols()
    cxx_names = {"cu_MAC_to_Regular4", "cu_Regular4_to_MAC", "SolveOpenPoissonRedBlackwithOccupy3D_MAC",
                 "SolveClosedPoissonRedBlackwithOccupy3D_MAC", "cu_MAC_to_Regular_vel"}
    c_names = declared - cxx_names
    assert set(capi.CAPI_SYMBOLS) | set(capi.LEGACY_C_SYMBOLS) == c_names
    for name in sorted(c_names):
        assert hasattr(zqs_lib, name), name
    for mangled in capi.LEGACY_CXX_SYMBOLS:
        assert hasattr(zqs_lib, mangled), mangled
    nm = shutil.which("nm")
    if nm:
        out = subprocess.run([nm, "-D", "--defined-only", str(capi.LIB_PATH)], capture_output=True, text=True).stdout
        for name in c_names:
            assert re.search(rf"\bT {name}$", out, re.M), name


def test_version_and_defaults(zqs_lib):
    assert zqs_lib.zqs_version() == 1
    p = capi.default_params(128, 128, 128)
    # ZQ_SmokeSimulationPara3D defaults (ZQ_SmokeSimulationUtils3D.cpp:18-72)
    assert p.substeps == 20 and abs(p.step_time - 0.01) < 1e-9 and p.buoyancy == 1.0 and p.tamb == 10.0
    assert p.sor_iters == 100 and p.omega == 1.0 and p.voxel_size == pytest.approx(1 / 128)
    assert p.n_sources == 1 and p.sources[0].shape == capi.SOURCE_BOX
    assert p.sources[0].cx == pytest.approx(64.0) and p.sources[0].temperature == 200.0


def test_params_struct_size_matches_c(tmp_path):
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("gcc missing")
    src = tmp_path / "sz.c"
    src.write_text('#include "zqs_capi.h"\n#include <stdio.h>\n#include <stddef.h>\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu\\n", sizeof(zqs_params), sizeof(zqs_source),'
                   ' sizeof(zqs_stats), sizeof(zqs_grid_layout), offsetof(zqs_params, sources));return 0;}\n')
    exe = tmp_path / "sz"
    subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", f"-I{INC}", str(src), "-o", str(exe)], check=True)
    vals = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert vals == [C.sizeof(capi.Params), C.sizeof(capi.Source), C.sizeof(capi.Stats), C.sizeof(capi.Layout),
                    capi.Params.sources.offset]


def test_legacy_header_compiles_as_cxx(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ missing")
    src = tmp_path / "leg.cpp"
    src.write_text('#include "zqs_legacy.h"\n'
                   'int main(){ using namespace ZQ_CUDA_Advection3D; return (int)ADV_VEL_INMAC_OUTMAC - 2 + '
                   '(int)ADV_SCA_REG - 2 + (int)ZQ_CUDA_AddForce3D::ADD_FORCE_SLICE - 1; }\n')
    subprocess.run([gxx, "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", f"-I{INC}",
                    "-I/usr/local/cuda/include", str(src)], check=True)


def test_enum_values_follow_reference_cuda_header():
    # ZQ_CUDA_Advection3D.h:7-21
    assert (capi.ADV_VEL_INREG_OUTREG, capi.ADV_VEL_INMAC_OUTMAC, capi.ADV_VEL_INREG_OUTMAC) == (0, 2, 4)
    assert (capi.ADV_SCA_MAC, capi.ADV_SCA_REG, capi.ADV_SCA_REG_BFECC) == (0, 2, 3)


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(FileNotFoundError):
        capi.load(tmp_path / "nope.so")


def test_added_structs_match_c(tmp_path):
    """zqs_object, zqs_camera and zqs_sor_variant as compiled C sees them."""
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("gcc missing")
    src = tmp_path / "sz2.c"
    src.write_text('#include "zqs_capi.h"\n#include <stdio.h>\n#include <stddef.h>\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu %zu\\n", sizeof(zqs_object), offsetof(zqs_object, vel),'
                   ' sizeof(zqs_camera), offsetof(zqs_camera, eye), offsetof(zqs_camera, steps),'
                   ' offsetof(zqs_camera, density_scale), sizeof(zqs_sor_variant));return 0;}\n')
    exe = tmp_path / "sz2"
    subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", f"-I{INC}", str(src), "-o", str(exe)], check=True)
    vals = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()]
    assert vals == [C.sizeof(capi.Object), capi.Object.vel.offset, C.sizeof(capi.Camera), capi.Camera.eye.offset,
                    capi.Camera.steps.offset, capi.Camera.density_scale.offset, C.sizeof(capi.SorVariant)]
