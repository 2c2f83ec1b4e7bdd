"""Pins of the CPU oracle and of the CUDA library to the reference's own kernels.

The reference's kernel files ZQ_CUDA_MACtoRegular.cu, ZQ_CUDA_Attenuation3D.cu,
ZQ_CUDA_AddForce3D.cu and ZQ_CUDA_Advection3D.cu are compiled unmodified
(oracle/build_ref.py) and run on the GPU with their host wrappers' launch
sequences restated (oracle/ref_kernels.py).  Their outputs are compared with
  * the FP32 oracle (oracle/), which restates them on the CPU, and
  * this library through its drop-in entry points (Attenuation3D, AddForce3D,
    Advect_Velocity, Advect_Scalar, cu_MAC_to_Regular4, cu_Regular4_to_MAC).

Two builds of the reference kernels run: "nofma" (-fmad=false, the arithmetic
contract the oracle and the library follow) must agree bit for bit wherever
the arithmetic is the reference's own; "default" (the reference's own build
flags, FP32 multiply-adds may be contracted) is held to relative L2 1e-6.

Advection: the reference samples through texture references, which CUDA 12
removed; oracle/ref_shim/texref_shim.cuh serves them from linear memory with
exact FP32 trilinear weights (the hardware's 9-bit weights cannot be
reproduced).  The kernels pass normalised coordinates, e.g. (x + 0.5)/(W + 1)
for the u texture; with power-of-two extents every normalisation of the cell
textures is exact, so the regular-grid modes (and the scalar reads) see the
oracle's texel coordinates and must match bit for bit; the MAC velocity
textures (extents W+1, H+1, D+1) carry a rounding of the normalisation, so the
MAC modes are held to the per-step tolerance of relative L2 1e-5.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2
from zq_smokesimulation_gb300 import capi
from zq_smokesimulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

TOL_DEFAULT_FLAGS = 1e-6   # reference built with its own flags (contracted FMAs)
TOL_MAC_TEX = 1e-5         # per-step tolerance: normalised MAC texture coordinates
VEL = ("u", "v", "w")
FORCE_DIMS = [(9, 11, 7), (16, 12, 10), (33, 17, 9), (64, 64, 64)]
POW2_DIMS = [(16, 8, 32), (32, 32, 32)]


@pytest.fixture(scope="module")
def ref():
    from oracle import ref_kernels
    out = {f: ref_kernels.RefKernels(f) for f in ("nofma", "default")}
    yield out
    for r in out.values():
        r.close()


def _state(w):
    return {k: np.ascontiguousarray(getattr(w, k), np.float32).copy() for k in ("u", "v", "w", "T", "rho")}


def _same(a, b, what):
    if not np.array_equal(a, b):
        bad = np.argwhere(a != b)
        raise AssertionError(f"{what}: {len(bad)} mismatches, first {bad[:3].tolist()}, "
                             f"{a[tuple(bad[0])]!r} vs {b[tuple(bad[0])]!r}, relL2 {rel_l2(a, b):.3e}")


def _case(dims, **kw):
    w = wl.small_case(*dims, vel_amp=0.3, **kw)
    w.params.gravity = 0.0   # the reference's force has no density term
    w.params.confine = 2.5   # make the confinement term large against buoyancy
    return w


# ------------------------------------------------------------- MAC <-> regular
@pytest.mark.parametrize("dims", FORCE_DIMS)
def test_mac_regular_pinned(zqs_lib, oracle32, ref, dims):
    """MAC_to_Regular4_Kernel, Regular4_to_MAC_{u,v,w}_Kernel (ZQ_CUDA_MACtoRegular.cu:9-99)."""
    import torch
    w = _case(dims)
    W, H, D = w.W, w.H, w.D
    st = _state(w)
    r4 = ref["nofma"].mac_to_regular4(W, H, D, st["u"], st["v"], st["w"])
    _same(r4, oracle32.mac_to_regular4(W, H, D, st["u"], st["v"], st["w"]), "MAC_to_Regular4 vs oracle")
    r4d = ref["default"].mac_to_regular4(W, H, D, st["u"], st["v"], st["w"])
    assert rel_l2(r4d, r4) <= TOL_DEFAULT_FLAGS
    back = ref["nofma"].regular4_to_mac(W, H, D, r4)
    ob = oracle32.regular4_to_mac(W, H, D, r4)
    for q in range(3):
        _same(back[q], ob[q], f"Regular4_to_MAC {VEL[q]} vs oracle")
    # the library's drop-in cu_MAC_to_Regular4 / cu_Regular4_to_MAC (device pointers)
    f_m2r = getattr(zqs_lib, capi.LEGACY_CXX_SYMBOLS[0])
    f_r2m = getattr(zqs_lib, capi.LEGACY_CXX_SYMBOLS[1])
    du, dv, dw = (torch.from_numpy(st[k]).cuda() for k in VEL)
    d4 = torch.zeros((D, H, W, 4), dtype=torch.float32, device="cuda")
    f_m2r(C.c_void_p(du.data_ptr()), C.c_void_p(dv.data_ptr()), C.c_void_p(dw.data_ptr()),
          C.c_void_p(d4.data_ptr()), W, H, D)
    torch.cuda.synchronize()
    _same(d4.cpu().numpy(), r4, "cu_MAC_to_Regular4 vs reference kernel")
    outs = [torch.zeros_like(t) for t in (du, dv, dw)]
    f_r2m(C.c_void_p(d4.data_ptr()), *(C.c_void_p(t.data_ptr()) for t in outs), W, H, D)
    torch.cuda.synchronize()
    for q in range(3):
        _same(outs[q].cpu().numpy(), back[q], f"cu_Regular4_to_MAC {VEL[q]} vs reference kernels")


# --------------------------------------------------------------- attenuation
@pytest.mark.parametrize("dims", FORCE_DIMS)
def test_attenuation_pinned(zqs_lib, oracle32, ref, dims):
    """Atten_{u,v,w}_Kernel, Atten_temperature_density_Kernel (ZQ_CUDA_Attenuation3D.cu:8-116)."""
    w = _case(dims)
    W, H, D = w.W, w.H, w.D
    fac = (0.93, 0.81, 0.67)
    out = {}
    for f in ("nofma", "default"):
        st = _state(w)
        ref[f].attenuation3d(W, H, D, st, w.occ, *fac)
        out[f] = st
    o = _state(w)
    p = w.params
    p.vel_atten, p.temp_atten, p.dens_atten = fac
    oracle32.attenuate(W, H, D, o, w.occ, p)
    g = _state(w)
    occ = np.ascontiguousarray(w.occ, np.uint8)
    ms = zqs_lib.Attenuation3D(*(g[k].ctypes.data for k in ("u", "v", "w", "T", "rho")), occ.ctypes.data, *fac,
                               W, H, D)
    assert ms >= 0, capi.last_error()
    for k in ("u", "v", "w", "T", "rho"):
        _same(out["nofma"][k], o[k], f"attenuation {k}: reference kernels vs oracle")
        _same(out["default"][k], o[k], f"attenuation {k}: reference (own flags) vs oracle")
        _same(g[k], out["nofma"][k], f"attenuation {k}: Attenuation3D vs reference kernels")


# --------------------------------------------------------------------- forces
@pytest.mark.parametrize("dims", FORCE_DIMS)
def test_add_force_pinned(zqs_lib, oracle32, ref, dims):
    """cu_AddForce3D's kernels (ZQ_CUDA_AddForce3D.cu:11-209, 387-420): vorticity,
    normalised gradient of its magnitude, confinement + buoyancy, face update."""
    w = _case(dims)
    W, H, D = w.W, w.H, w.D
    p = w.params
    args = (float(p.voxel_size), float(p.step_time), float(p.buoyancy), float(p.confine), float(p.tamb))
    out, tmp = {}, {}
    for f in ("nofma", "default"):
        st = _state(w)
        tmp[f] = ref[f].add_force3d(W, H, D, st, w.occ, *args)
        out[f] = st
    # the oracle's intermediates and result
    vort, vs = oracle32.vorticity(W, H, D, w.u, w.v, w.w, p.voxel_size)
    _same(tmp["nofma"]["vort"], vort, "vortVector vs oracle")
    _same(tmp["nofma"]["vs"], vs, "vortScale vs oracle")
    o = _state(w)
    oracle32.add_force(W, H, D, o, w.occ, p)
    for k in VEL:
        _same(out["nofma"][k], o[k], f"add_force {k}: reference kernels vs oracle")
        assert rel_l2(out["default"][k], o[k]) <= TOL_DEFAULT_FLAGS, k
    assert max(float(np.abs(out["nofma"][k] - getattr(w, k)).max()) for k in VEL) > 0.0  # forces acted
    # the library's drop-in AddForce3D
    g = _state(w)
    occ = np.ascontiguousarray(w.occ, np.uint8)
    ms = zqs_lib.AddForce3D(g["u"].ctypes.data, g["v"].ctypes.data, g["w"].ctypes.data, occ.ctypes.data,
                            g["T"].ctypes.data, *args, W, H, D, 0)
    assert ms >= 0, capi.last_error()
    for k in VEL:
        _same(g[k], out["nofma"][k], f"AddForce3D {k} vs reference kernels")


# ------------------------------------------------------------------ advection
VMODES = [capi.ADV_VEL_INREG_OUTREG, capi.ADV_VEL_INREG_OUTREG_BFECC, capi.ADV_VEL_INMAC_OUTMAC,
          capi.ADV_VEL_INMAC_OUTMAC_BFECC, capi.ADV_VEL_INREG_OUTMAC, capi.ADV_VEL_INREG_OUTMAC_BFECC]
REGULAR_VMODES = {capi.ADV_VEL_INREG_OUTREG, capi.ADV_VEL_INREG_OUTREG_BFECC}


def _adv_case(dims, closed=False, substeps=5):
    w = _case(dims, closed=closed, substeps=substeps)
    w.params.step_time = 0.5   # backtraces of a few cells
    return w


def _dt_sub(p):
    return np.float32(np.float32(p.step_time) / np.float32(p.substeps))


@pytest.mark.parametrize("dims", POW2_DIMS)
@pytest.mark.parametrize("mode", VMODES)
@pytest.mark.parametrize("is_open", [True, False])
def test_advect_velocity_pinned(zqs_lib, oracle32, ref, dims, mode, is_open):
    """Advect_Velocity's six modes (ZQ_CUDA_Advection3D.cu:76-377, 471-650,
    1061-1474) with the open and closed write-backs."""
    w = _adv_case(dims, closed=not is_open)
    W, H, D = w.W, w.H, w.D
    p = w.params
    dts = _dt_sub(p)
    res = {}
    for f in ("nofma", "default"):
        r = ref[f]
        r.prepare_advection(W, H, D, p.voxel_size, p.substeps, dts)
        st = _state(w)
        r.advect_velocity(st, w.occ, is_open, mode)
        res[f] = st
    o = _state(w)
    rc = oracle32.advect_velocity(W, H, D, o, w.occ, p, mode, is_open)
    assert rc == 0
    zqs_lib.ZQ_Cuda_Prepare_Advection(W, H, D, float(p.voxel_size), p.substeps, float(dts))
    g = _state(w)
    occ = np.ascontiguousarray(w.occ, np.uint8)
    ms = zqs_lib.Advect_Velocity(g["u"].ctypes.data, g["v"].ctypes.data, g["w"].ctypes.data, occ.ctypes.data,
                                 is_open, mode)
    assert ms >= 0, capi.last_error()
    moved = max(float(np.abs(res["nofma"][k] - getattr(w, k)).max()) for k in VEL)
    assert moved > 0.0
    for k in VEL:
        _same(g[k], o[k], f"Advect_Velocity {k} vs oracle")
        if mode in REGULAR_VMODES:
            _same(res["nofma"][k], o[k], f"mode {mode} {k}: reference kernels vs oracle")
        else:
            assert rel_l2(res["nofma"][k], o[k]) <= TOL_MAC_TEX, (k, rel_l2(res["nofma"][k], o[k]))
        assert rel_l2(res["default"][k], res["nofma"][k]) <= TOL_DEFAULT_FLAGS, k


SMODES = [capi.ADV_SCA_MAC, capi.ADV_SCA_MAC_BFECC, capi.ADV_SCA_REG, capi.ADV_SCA_REG_BFECC]


@pytest.mark.parametrize("dims", POW2_DIMS + [(64, 64, 64)])
@pytest.mark.parametrize("mode", SMODES)
def test_advect_scalar_pinned(zqs_lib, oracle32, ref, dims, mode):
    """Advect_Scalar's kernels and the cu_Advect_Scalar_* sequences
    (ZQ_CUDA_Advection3D.cu:379-469, 1476-1648; the BFECC sequences are the
    ones the reference's entry point never reaches)."""
    w = _adv_case(dims)
    W, H, D = w.W, w.H, w.D
    p = w.params
    dts = _dt_sub(p)
    res = {}
    for f in ("nofma", "default"):
        r = ref[f]
        r.prepare_advection(W, H, D, p.voxel_size, p.substeps, dts)
        res[f] = r.advect_scalar(_state(w), w.occ, mode)
    o = _state(w)
    rc = oracle32.advect_scalar(W, H, D, o, w.occ, p, mode)
    assert rc == 0
    zqs_lib.ZQ_Cuda_Prepare_Advection(W, H, D, float(p.voxel_size), p.substeps, float(dts))
    g = _state(w)
    occ = np.ascontiguousarray(w.occ, np.uint8)
    oT, oD = np.empty_like(g["T"]), np.empty_like(g["rho"])
    ms = zqs_lib.Advect_Scalar(g["u"].ctypes.data, g["v"].ctypes.data, g["w"].ctypes.data, occ.ctypes.data,
                               g["T"].ctypes.data, g["rho"].ctypes.data, oT.ctypes.data, oD.ctypes.data, mode)
    assert ms >= 0, capi.last_error()
    for name, a, b in (("T", oT, o["T"]), ("rho", oD, o["rho"])):
        _same(a, b, f"Advect_Scalar {name} vs oracle")
    for q, name in enumerate(("T", "rho")):
        rn = res["nofma"][q]
        if mode in (capi.ADV_SCA_REG, capi.ADV_SCA_REG_BFECC):
            _same(rn, o[name], f"scalar mode {mode} {name}: reference kernels vs oracle")
        else:
            assert rel_l2(rn, o[name]) <= TOL_MAC_TEX, (name, rel_l2(rn, o[name]))
        assert rel_l2(res["default"][q], rn) <= TOL_DEFAULT_FLAGS, name
        assert not np.array_equal(rn, getattr(w, name))
