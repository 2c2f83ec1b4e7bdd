"""The reference's own CUDA kernels, run on this GPU (TEST INFRASTRUCTURE ONLY).

Loads the device-only modules that oracle/build_ref.py compiles from the
reference's unmodified kernel files (ZQ_CUDA_MACtoRegular.cu,
ZQ_CUDA_Attenuation3D.cu, ZQ_CUDA_AddForce3D.cu, ZQ_CUDA_Advection3D.cu) and
launches them through the CUDA driver API (ctypes on libcuda).  The host
wrappers of the reference are restated here launch by launch, with the same
grids (BLOCK_SIZE 16), the same kernel order and the same zero-filled
temporaries, each citing the lines it follows.  Only the tests import this
module, to pin the CPU oracle and the CUDA library to the reference's own
kernels; nothing in the product loads it.

Deviations forced by the build environment, each stated where it applies:
  * cu_AddForce3D's cell-centre velocity comes from ZQlibCuda's
    cu_MAC_to_Regular_vel (not in the reference tree); it is formed here with
    the reference's MAC_to_Regular4_Kernel and split into three arrays.
  * The whole-z AddForce_w_Kernel (ZQ_CUDA_AddForce3D.cu:360-385) reads
    occupy[-1 plane] at z = 0 and is never launched; its per-slice form
    (:387-420, launched for z = 0..D as cu_AddForce_u_v_w2 does, :502-506)
    gives the intended result.
  * Texture references are emulated by oracle/ref_shim/texref_shim.cuh: a
    bind snapshots the data (as cudaMemcpy3D into a cudaArray does) and
    tex3D interpolates exactly in FP32 instead of with 9-bit weights.

Device memory comes from torch (plumbing only); arrays cross as numpy.
"""
from __future__ import annotations

import ctypes as C
import struct
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BS = 16  # BLOCK_SIZE of the reference's thread blocks

# cudaTextureFilterMode / cudaTextureAddressMode values (driver_types.h)
_FILTER_POINT, _FILTER_LINEAR = 0, 1
_ADDR_CLAMP = 1

_N_ADV = "ZQ_CUDA_Advection3D"


def _mangle_ns(ns: str, name: str, sig: str = "") -> str:
    return f"_ZN{len(ns)}{ns}{len(name)}{name}E{sig}"


# kernel symbols (Itanium C++ mangling of the reference's declarations)
_K = {
    "mac2reg": ("mac", _mangle_ns("ZQ_CUDA_MACtoRegular", "MAC_to_Regular4_Kernel", "PKfS1_S1_P6float4iii")),
    "reg2mac_u": ("mac", _mangle_ns("ZQ_CUDA_MACtoRegular", "Regular4_to_MAC_u_Kernel", "PK6float4Pfiii")),
    "reg2mac_v": ("mac", _mangle_ns("ZQ_CUDA_MACtoRegular", "Regular4_to_MAC_v_Kernel", "PK6float4Pfiii")),
    "reg2mac_w": ("mac", _mangle_ns("ZQ_CUDA_MACtoRegular", "Regular4_to_MAC_w_Kernel", "PK6float4Pfiii")),
    "atten_u": ("atten", _mangle_ns("ZQ_CUDA_Attenuation3D", "Atten_u_Kernel", "PfPKbfiii")),
    "atten_v": ("atten", _mangle_ns("ZQ_CUDA_Attenuation3D", "Atten_v_Kernel", "PfPKbfiii")),
    "atten_w": ("atten", _mangle_ns("ZQ_CUDA_Attenuation3D", "Atten_w_Kernel", "PfPKbfiii")),
    "atten_td": ("atten", _mangle_ns("ZQ_CUDA_Attenuation3D", "Atten_temperature_density_Kernel", "PfS0_ffiii")),
    "vort": ("force", _mangle_ns("ZQ_CUDA_AddForce3D", "Compute_Vorticity_Vector_Scale_Kernel", "PfS0_PKfS2_S2_fiii")),
    "gradvort": ("force", _mangle_ns("ZQ_CUDA_AddForce3D", "Compute_Gradient_of_VorticityScale_Kernel", "PfS0_iii")),
    "force": ("force", _mangle_ns("ZQ_CUDA_AddForce3D", "Compute_Force_Kernel", "PfPKfS2_S2_ffffiii")),
    "addforce_u": ("force", _mangle_ns("ZQ_CUDA_AddForce3D", "AddForce_u_Kernel", "PfPKbPKffiii")),
    "addforce_v": ("force", _mangle_ns("ZQ_CUDA_AddForce3D", "AddForce_v_Kernel", "PfPKbPKffiii")),
    "addforce_w_slice": ("force", _mangle_ns("ZQ_CUDA_AddForce3D", "AddForce_w_Kernel", "iPfPKbPKffiii")),
    "neg": ("advect", _mangle_ns(_N_ADV, "Velocity_Negative_Kernel", "Pfi")),
    "neg4": ("advect", _mangle_ns(_N_ADV, "Velocity_Negative_4channels_Kernel", "P6float4i")),
    "inc": ("advect", _mangle_ns(_N_ADV, "Input_Increment_Kernel", "PfPKfi")),
    "inc4": ("advect", _mangle_ns(_N_ADV, "Input_Increment_4channels_Kernel", "P6float4PKS0_i")),
    "adv_regreg": ("advect", _mangle_ns(_N_ADV, "Advect_Velocity_inRegular_outRegular_Kernel", "P6float4")),
    "adv_regmac_u": ("advect", _mangle_ns(_N_ADV, "Advect_Velocity_inRegular_outMAC_u_Kernel", "Pf")),
    "adv_regmac_v": ("advect", _mangle_ns(_N_ADV, "Advect_Velocity_inRegular_outMAC_v_Kernel", "Pf")),
    "adv_regmac_w": ("advect", _mangle_ns(_N_ADV, "Advect_Velocity_inRegular_outMAC_w_Kernel", "Pf")),
    "adv_macmac_u": ("advect", _mangle_ns(_N_ADV, "Advect_Velocity_inMAC_outMAC_u_Kernel", "Pf")),
    "adv_macmac_v": ("advect", _mangle_ns(_N_ADV, "Advect_Velocity_inMAC_outMAC_v_Kernel", "Pf")),
    "adv_macmac_w": ("advect", _mangle_ns(_N_ADV, "Advect_Velocity_inMAC_outMAC_w_Kernel", "Pf")),
    "adv_sca_reg": ("advect", _mangle_ns(_N_ADV, "Advect_Scalar_Regular_Velocity_Kernel", "PfS0_")),
    "adv_sca_mac": ("advect", _mangle_ns(_N_ADV, "Advect_Scalar_MAC_Velocity_Kernel", "PfS0_")),
    "apply_open_u": ("advect", _mangle_ns(_N_ADV, "Apply_Advect_Velocity_Result_Open_u_Kernel", "PKfPKbPfiii")),
    "apply_open_v": ("advect", _mangle_ns(_N_ADV, "Apply_Advect_Velocity_Result_Open_v_Kernel", "PKfPKbPfiii")),
    "apply_open_w": ("advect", _mangle_ns(_N_ADV, "Apply_Advect_Velocity_Result_Open_w_Kernel", "PKfPKbPfiii")),
    "apply_closed_u": ("advect", _mangle_ns(_N_ADV, "Apply_Advect_Velocity_Result_Closed_u_Kernel", "PKfPKbPfiii")),
    "apply_closed_v": ("advect", _mangle_ns(_N_ADV, "Apply_Advect_Velocity_Result_Closed_v_Kernel", "PKfPKbPfiii")),
    "apply_closed_w": ("advect", _mangle_ns(_N_ADV, "Apply_Advect_Velocity_Result_Closed_w_Kernel", "PKfPKbPfiii")),
}
# texture references (ZQ_CUDA_Advection3D.cu:10-20) and constants (:29-34)
_TEX = ("tex_velocity_regular", "tex_velocity_MAC_u", "tex_velocity_MAC_v", "tex_velocity_MAC_w", "tex_occupy",
        "tex_inputVelocity_MAC_u", "tex_inputVelocity_MAC_v", "tex_inputVelocity_MAC_w",
        "tex_inputVelocity_regular", "tex_temperature", "tex_density")
_TEX_BYTES = 48  # sizeof(zq_texref<...>) in texref_shim.cuh

# AdvectVelocityType / AdvectScalarType (ZQ_CUDA_Advection3D.h:7-21)
INREG_OUTREG, INREG_OUTREG_BFECC, INMAC_OUTMAC, INMAC_OUTMAC_BFECC, INREG_OUTMAC, INREG_OUTMAC_BFECC = range(6)
SCA_MAC, SCA_MAC_BFECC, SCA_REG, SCA_REG_BFECC = range(4)


def available() -> bool:
    from . import build_ref
    return build_ref.available()


class _Driver:
    def __init__(self):
        self.lib = C.CDLL("libcuda.so.1")
        L = self.lib
        L.cuGetErrorString.argtypes = [C.c_int, C.POINTER(C.c_char_p)]
        L.cuModuleLoadData.argtypes = [C.POINTER(C.c_void_p), C.c_void_p]
        L.cuModuleGetFunction.argtypes = [C.POINTER(C.c_void_p), C.c_void_p, C.c_char_p]
        L.cuModuleGetGlobal_v2.argtypes = [C.POINTER(C.c_uint64), C.POINTER(C.c_size_t), C.c_void_p, C.c_char_p]
        L.cuLaunchKernel.argtypes = [C.c_void_p] + [C.c_uint] * 7 + [C.c_void_p, C.POINTER(C.c_void_p),
                                                                     C.POINTER(C.c_void_p)]
        L.cuMemcpyHtoD_v2.argtypes = [C.c_uint64, C.c_void_p, C.c_size_t]
        L.cuCtxGetCurrent.argtypes = [C.POINTER(C.c_void_p)]
        L.cuModuleUnload.argtypes = [C.c_void_p]

    def check(self, rc: int, what: str):
        if rc != 0:
            s = C.c_char_p()
            self.lib.cuGetErrorString(rc, C.byref(s))
            raise RuntimeError(f"{what}: CUDA driver error {rc} ({(s.value or b'?').decode()})")


class RefKernels:
    """The reference's kernels in one flavour ("nofma": -fmad=false, the
    oracle's arithmetic contract; "default": the reference's own build flags)."""

    def __init__(self, flavour: str = "nofma"):
        import torch
        from . import build_ref
        if not build_ref.available():
            raise RuntimeError("reference modules missing: build them with oracle/build_ref.py where the "
                               "reference checkout exists")
        self.torch = torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # make the primary context current on this thread
        self.drv = _Driver()
        ctx = C.c_void_p()
        self.drv.check(self.drv.lib.cuCtxGetCurrent(C.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        self.mods = {}
        self._img = {}
        for name in build_ref.MODULES:
            data = build_ref.module_path(name, flavour).read_bytes()
            buf = C.create_string_buffer(data, len(data))
            self._img[name] = buf
            m = C.c_void_p()
            self.drv.check(self.drv.lib.cuModuleLoadData(C.byref(m), buf), f"load {name}.{flavour}")
            self.mods[name] = m
        self.fns = {}
        for key, (mod, sym) in _K.items():
            f = C.c_void_p()
            self.drv.check(self.drv.lib.cuModuleGetFunction(C.byref(f), self.mods[mod], sym.encode()), sym)
            self.fns[key] = f
        self._tex_keep: dict[str, object] = {}
        self.dims = None

    def close(self):
        self.torch.cuda.synchronize()
        for m in self.mods.values():
            self.drv.lib.cuModuleUnload(m)
        self.mods.clear()
        self._tex_keep.clear()

    # -- plumbing -------------------------------------------------------------
    def dev(self, a: np.ndarray):
        t = self.torch.from_numpy(np.ascontiguousarray(a))
        return t.to("cuda")

    def zeros(self, shape, dtype=np.float32):
        td = {np.float32: self.torch.float32, np.uint8: self.torch.uint8}[np.dtype(dtype).type]
        return self.torch.zeros(tuple(shape), dtype=td, device="cuda")

    @staticmethod
    def host(t) -> np.ndarray:
        return t.cpu().numpy().copy()

    def launch(self, key: str, grid, block, *args):
        vals = []
        for a in args:
            if hasattr(a, "data_ptr"):
                vals.append(C.c_void_p(a.data_ptr()))
            elif isinstance(a, float):
                vals.append(C.c_float(a))
            elif isinstance(a, np.float32):
                vals.append(C.c_float(float(a)))
            elif isinstance(a, (int, np.integer)):
                vals.append(C.c_int(int(a)))
            else:
                raise TypeError(type(a))
        arr = (C.c_void_p * max(1, len(vals)))(*[C.cast(C.pointer(v), C.c_void_p) for v in vals])
        g = tuple(grid) + (1,) * (3 - len(grid))
        b = tuple(block) + (1,) * (3 - len(block))
        stream = self.torch.cuda.current_stream().cuda_stream
        rc = self.drv.lib.cuLaunchKernel(self.fns[key], g[0], g[1], g[2], b[0], b[1], b[2], 0, C.c_void_p(stream),
                                         arr, None)
        self.drv.check(rc, key)

    def _global(self, mod: str, name: str):
        p = C.c_uint64()
        n = C.c_size_t()
        sym = _mangle_ns(_N_ADV, name) if mod == "advect" else name
        self.drv.check(self.drv.lib.cuModuleGetGlobal_v2(C.byref(p), C.byref(n), self.mods[mod], sym.encode()), sym)
        return p.value, n.value

    def _set_global(self, mod: str, name: str, data: bytes):
        addr, n = self._global(mod, name)
        if n != len(data):
            raise RuntimeError(f"{name}: {n} bytes in the module, {len(data)} given")
        self.torch.cuda.synchronize()  # kernels in flight may still read the old value
        self.drv.check(self.drv.lib.cuMemcpyHtoD_v2(addr, data, len(data)), f"set {name}")

    # -- ZQ_CUDA_MACtoRegular.cu:101-120 ---------------------------------------
    def grid2(self, nx, ny):
        return ((nx + BS - 1) // BS, (ny + BS - 1) // BS)

    def mac_to_regular4_dev(self, u, v, w, W, H, D):
        vel = self.zeros((D, H, W, 4))
        self.launch("mac2reg", self.grid2(W, H), (BS, BS), u, v, w, vel, W, H, D)
        return vel

    def regular4_to_mac_dev(self, vel, u, v, w, W, H, D):
        self.launch("reg2mac_u", self.grid2(W + 1, H), (BS, BS), vel, u, W, H, D)
        self.launch("reg2mac_v", self.grid2(W, H + 1), (BS, BS), vel, v, W, H, D)
        self.launch("reg2mac_w", self.grid2(W, H), (BS, BS), vel, w, W, H, D)

    def mac_to_regular4(self, W, H, D, u, v, w) -> np.ndarray:
        return self.host(self.mac_to_regular4_dev(self.dev(u), self.dev(v), self.dev(w), W, H, D))

    def regular4_to_mac(self, W, H, D, vel4):
        u, v, w = self.zeros((D, H, W + 1)), self.zeros((D, H + 1, W)), self.zeros((D + 1, H, W))
        self.regular4_to_mac_dev(self.dev(np.asarray(vel4, np.float32)), u, v, w, W, H, D)
        return self.host(u), self.host(v), self.host(w)

    # -- cu_Attenuation3D, ZQ_CUDA_Attenuation3D.cu:118-136 ------------------------
    def attenuation3d(self, W, H, D, st, occ, vel_atten, temp_atten, dens_atten):
        """In place on st's u, v, w, T, rho (numpy)."""
        d = {k: self.dev(st[k]) for k in ("u", "v", "w", "T", "rho")}
        o = self.dev(np.ascontiguousarray(occ, np.uint8))
        va, ta, da = np.float32(vel_atten), np.float32(temp_atten), np.float32(dens_atten)
        self.launch("atten_u", self.grid2(W + 1, H), (BS, BS), d["u"], o, va, W, H, D)
        self.launch("atten_v", self.grid2(W, H + 1), (BS, BS), d["v"], o, va, W, H, D)
        self.launch("atten_w", self.grid2(W, H), (BS, BS), d["w"], o, va, W, H, D)
        self.launch("atten_td", self.grid2(W, H), (BS, BS), d["T"], d["rho"], ta, da, W, H, D)
        for k in d:
            st[k][...] = self.host(d[k])

    # -- cu_AddForce3D, ZQ_CUDA_AddForce3D.cu:510-556 ------------------------------
    def add_force3d(self, W, H, D, st, occ, deltah, deltat, buoy, confine, tamb):
        """In place on st's u, v, w (numpy); returns the temporaries
        (vortVector, vortScale, gradVort, force) as numpy arrays."""
        n = W * H * D
        mu, mv, mw = self.dev(st["u"]), self.dev(st["v"]), self.dev(st["w"])
        T = self.dev(np.ascontiguousarray(st["T"], np.float32))
        o = self.dev(np.ascontiguousarray(occ, np.uint8))
        # cell-centre velocity (cu_MAC_to_Regular_vel, :523) via MAC_to_Regular4_Kernel
        vel4 = self.mac_to_regular4_dev(mu, mv, mw, W, H, D)
        cu, cv, cw = (vel4[..., q].contiguous() for q in range(3))
        vort, vs = self.zeros((n * 3,)), self.zeros((n,))   # cudaMemset 0, :527-530
        grad, force = self.zeros((n * 3,)), self.zeros((n * 3,))   # :535-536, :541-542
        h, dt = np.float32(deltah), np.float32(deltat)
        g = self.grid2(W, H)
        self.launch("vort", g, (BS, BS), vort, vs, cu, cv, cw, h, W, H, D)                       # :429-431
        self.launch("gradvort", g, (BS, BS), grad, vs, W, H, D)                                   # :442-448
        self.launch("force", g, (BS, BS), force, grad, vort, T, np.float32(confine), np.float32(buoy), h,
                    np.float32(tamb), W, H, D)                                                    # :460-467
        self.launch("addforce_u", self.grid2(W + 1, H), (BS, BS), mu, o, force, dt, W, H, D)      # :479
        self.launch("addforce_v", self.grid2(W, H + 1), (BS, BS), mv, o, force, dt, W, H, D)      # :480
        for z in range(D + 1):                                                                    # :505-506
            self.launch("addforce_w_slice", g, (BS, BS), z, mw, o, force, dt, W, H, D)
        for k, t in (("u", mu), ("v", mv), ("w", mw)):
            st[k][...] = self.host(t)
        return {"vort": self.host(vort).reshape(D, H, W, 3), "vs": self.host(vs).reshape(D, H, W),
                "grad": self.host(grad).reshape(D, H, W, 3), "force": self.host(force).reshape(D, H, W, 3)}

    # -- advection: ZQ_Cuda_Prepare_Advection, ZQ_CUDA_Advection3D.cu:1652-1668 ----
    def prepare_advection(self, W, H, D, voxel_size, steps, deltatt):
        self.dims = (W, H, D)
        for name, val in (("d_width", W), ("d_height", H), ("d_depth", D), ("d_steps", steps)):
            self._set_global("advect", name, struct.pack("<I", int(val)))
        self._set_global("advect", "d_voxelSize", struct.pack("<f", float(np.float32(voxel_size))))
        self._set_global("advect", "d_deltatt", struct.pack("<f", float(np.float32(deltatt))))

    def _bind(self, tex: str, src, nx, ny, nz, linear=True):
        """cu_Copy_to_tex_* (Adv3D:654-993): a snapshot of src bound with
        normalised coordinates, clamp addressing, linear (point for occupancy)."""
        snap = src.clone().contiguous()
        self._tex_keep[tex] = snap
        data = struct.pack("<iiiiiiQiiii", 1, _FILTER_LINEAR if linear else _FILTER_POINT, _ADDR_CLAMP, _ADDR_CLAMP,
                           _ADDR_CLAMP, 1 if linear else 0, snap.data_ptr(), nx, ny, nz, 0)
        assert len(data) == _TEX_BYTES
        self._set_global("advect", tex, data)

    def _bind_mac_vel(self, u, v, w):
        W, H, D = self.dims
        self._bind("tex_velocity_MAC_u", u, W + 1, H, D)
        self._bind("tex_velocity_MAC_v", v, W, H + 1, D)
        self._bind("tex_velocity_MAC_w", w, W, H, D + 1)

    def _bind_mac_input(self, u, v, w):
        W, H, D = self.dims
        self._bind("tex_inputVelocity_MAC_u", u, W + 1, H, D)
        self._bind("tex_inputVelocity_MAC_v", v, W, H + 1, D)
        self._bind("tex_inputVelocity_MAC_w", w, W, H, D + 1)

    def _neg(self, u, v, w):  # cu_Velocity_Negative, Adv3D:997-1010
        for t in (u, v, w):
            n = t.numel()
            self.launch("neg", ((n + BS * BS - 1) // (BS * BS),), (BS * BS,), t, n)

    def _neg4(self, vel):  # cu_Velocity_Negative_4channels, Adv3D:1012-1019
        n = vel.numel() // 4
        self.launch("neg4", ((n + BS * BS - 1) // (BS * BS),), (BS * BS,), vel, n)

    def _inc(self, a, b):  # cu_Input_Increment, Adv3D:1021-1027
        n = a.numel()
        self.launch("inc", ((n + BS * BS - 1) // (BS * BS),), (BS * BS,), a, b, n)

    def _inc4(self, a, b):  # cu_Input_Increment_4channels, Adv3D:1029-1035
        n = a.numel() // 4
        self.launch("inc4", ((n + BS * BS - 1) // (BS * BS),), (BS * BS,), a, b, n)

    def _faces3(self, prefix, ou, ov, ow):
        W, H, D = self.dims
        self.launch(prefix + "_u", self.grid2(W + 1, H), (BS, BS), ou)
        self.launch(prefix + "_v", self.grid2(W, H + 1), (BS, BS), ov)
        self.launch(prefix + "_w", self.grid2(W, H), (BS, BS), ow)

    def _apply(self, is_open, ou, ov, ow, occ, u, v, w):  # Adv3D:1037-1059
        W, H, D = self.dims
        k = "apply_open" if is_open else "apply_closed"
        self.launch(k + "_u", self.grid2(W + 1, H), (BS, BS), ou, occ, u, W, H, D)
        self.launch(k + "_v", self.grid2(W, H + 1), (BS, BS), ov, occ, v, W, H, D)
        self.launch(k + "_w", self.grid2(W, H), (BS, BS), ow, occ, w, W, H, D)

    def _out_mac(self):
        W, H, D = self.dims
        return self.zeros((D, H, W + 1)), self.zeros((D, H + 1, W)), self.zeros((D + 1, H, W))

    def advect_velocity(self, st, occ, is_open, mode):
        """Advect_Velocity's device part (Adv3D:1713-1732) for `mode`, in place
        on st's u, v, w (numpy)."""
        W, H, D = self.dims
        u, v, w = self.dev(st["u"]), self.dev(st["v"]), self.dev(st["w"])
        o = self.dev(np.ascontiguousarray(occ, np.uint8))
        self._bind("tex_occupy", o, W, H, D, linear=False)
        g = self.grid2(W, H)
        if mode == INMAC_OUTMAC:  # Adv3D:1184-1238
            self._bind_mac_vel(u, v, w)
            self._bind_mac_input(u, v, w)
            ou, ov, ow = self._out_mac()
            self._faces3("adv_macmac", ou, ov, ow)
            self._apply(is_open, ou, ov, ow, o, u, v, w)
        elif mode == INMAC_OUTMAC_BFECC:  # Adv3D:1240-1336
            self._bind_mac_vel(u, v, w)
            self._bind_mac_input(u, v, w)
            ou, ov, ow = self._out_mac()
            self._faces3("adv_macmac", ou, ov, ow)
            self._neg(u, v, w)
            self._bind_mac_vel(u, v, w)
            self._bind_mac_input(ou, ov, ow)
            self._faces3("adv_macmac", ou, ov, ow)
            self._neg(u, v, w)
            self._bind_mac_vel(u, v, w)
            self._inc(u, ou)
            self._inc(v, ov)
            self._inc(w, ow)
            self._bind_mac_input(u, v, w)
            self._faces3("adv_macmac", ou, ov, ow)
            self._apply(is_open, ou, ov, ow, o, u, v, w)
        elif mode == INREG_OUTREG:  # Adv3D:1061-1108
            vel = self.mac_to_regular4_dev(u, v, w, W, H, D)
            self._bind("tex_velocity_regular", vel, W, H, D)
            self._bind("tex_inputVelocity_regular", vel, W, H, D)
            self.launch("adv_regreg", g, (BS, BS), vel)
            ou, ov, ow = self._out_mac()
            self.regular4_to_mac_dev(vel, ou, ov, ow, W, H, D)
            self._apply(is_open, ou, ov, ow, o, u, v, w)
        elif mode == INREG_OUTREG_BFECC:  # Adv3D:1110-1182
            vel = self.mac_to_regular4_dev(u, v, w, W, H, D)
            io = self.zeros((D, H, W, 4))
            self._bind("tex_velocity_regular", vel, W, H, D)
            self._bind("tex_inputVelocity_regular", vel, W, H, D)
            self.launch("adv_regreg", g, (BS, BS), io)
            self._neg4(vel)
            self._bind("tex_velocity_regular", vel, W, H, D)
            self._bind("tex_inputVelocity_regular", io, W, H, D)
            self.launch("adv_regreg", g, (BS, BS), io)
            self._neg4(vel)
            self._bind("tex_velocity_regular", vel, W, H, D)
            self._inc4(vel, io)
            self._bind("tex_inputVelocity_regular", vel, W, H, D)
            self.launch("adv_regreg", g, (BS, BS), io)
            ou, ov, ow = self._out_mac()
            self.regular4_to_mac_dev(io, ou, ov, ow, W, H, D)
            self._apply(is_open, ou, ov, ow, o, u, v, w)
        elif mode == INREG_OUTMAC:  # Adv3D:1338-1387
            vel = self.mac_to_regular4_dev(u, v, w, W, H, D)
            self._bind("tex_velocity_regular", vel, W, H, D)
            self._bind("tex_inputVelocity_regular", vel, W, H, D)
            ou, ov, ow = self._out_mac()
            self._faces3("adv_regmac", ou, ov, ow)
            self._apply(is_open, ou, ov, ow, o, u, v, w)
        elif mode == INREG_OUTMAC_BFECC:  # Adv3D:1389-1474
            vel = self.mac_to_regular4_dev(u, v, w, W, H, D)
            self._bind("tex_velocity_regular", vel, W, H, D)
            self._bind("tex_inputVelocity_regular", vel, W, H, D)
            ou, ov, ow = self._out_mac()
            self._faces3("adv_regmac", ou, ov, ow)
            io = self.mac_to_regular4_dev(ou, ov, ow, W, H, D)
            self._neg4(vel)
            self._bind("tex_velocity_regular", vel, W, H, D)
            self._bind("tex_inputVelocity_regular", io, W, H, D)
            self._faces3("adv_regmac", ou, ov, ow)
            io = self.mac_to_regular4_dev(ou, ov, ow, W, H, D)
            self._neg4(vel)
            self._bind("tex_velocity_regular", vel, W, H, D)
            self._inc4(vel, io)
            self._bind("tex_inputVelocity_regular", vel, W, H, D)
            self._faces3("adv_regmac", ou, ov, ow)
            self._apply(is_open, ou, ov, ow, o, u, v, w)
        else:
            raise ValueError(mode)
        self.torch.cuda.synchronize()
        for k, t in (("u", u), ("v", v), ("w", w)):
            st[k][...] = self.host(t)

    def advect_scalar(self, st, occ, mode):
        """cu_Advect_Scalar_* (Adv3D:1476-1648) for `mode`; returns (T, rho)
        (numpy).  The BFECC forms overwrite their input copies as the
        reference's do; st is not modified."""
        W, H, D = self.dims
        u, v, w = self.dev(st["u"]), self.dev(st["v"]), self.dev(st["w"])
        o = self.dev(np.ascontiguousarray(occ, np.uint8))
        iT, iD = self.dev(st["T"]), self.dev(st["rho"])
        oT, oD = self.zeros((D, H, W)), self.zeros((D, H, W))
        g = self.grid2(W, H)
        self._bind("tex_occupy", o, W, H, D, linear=False)
        if mode in (SCA_REG, SCA_REG_BFECC):  # Adv3D:1476-1560
            vel = self.mac_to_regular4_dev(u, v, w, W, H, D)
            self._bind("tex_velocity_regular", vel, W, H, D)
            self._bind("tex_temperature", iT, W, H, D)
            self._bind("tex_density", iD, W, H, D)
            self.launch("adv_sca_reg", g, (BS, BS), oT, oD)
            if mode == SCA_REG_BFECC:
                self._neg4(vel)
                self._bind("tex_velocity_regular", vel, W, H, D)
                self._bind("tex_temperature", oT, W, H, D)
                self._bind("tex_density", oD, W, H, D)
                self.launch("adv_sca_reg", g, (BS, BS), oT, oD)
                self._neg4(vel)
                self._bind("tex_velocity_regular", vel, W, H, D)
                self._inc(iT, oT)
                self._inc(iD, oD)
                self._bind("tex_temperature", iT, W, H, D)
                self._bind("tex_density", iD, W, H, D)
                self.launch("adv_sca_reg", g, (BS, BS), oT, oD)
        elif mode in (SCA_MAC, SCA_MAC_BFECC):  # Adv3D:1562-1648
            self._bind_mac_vel(u, v, w)
            self._bind("tex_temperature", iT, W, H, D)
            self._bind("tex_density", iD, W, H, D)
            self.launch("adv_sca_mac", g, (BS, BS), oT, oD)
            if mode == SCA_MAC_BFECC:
                self._neg(u, v, w)
                self._bind_mac_vel(u, v, w)
                self._bind("tex_temperature", oT, W, H, D)
                self._bind("tex_density", oD, W, H, D)
                self.launch("adv_sca_mac", g, (BS, BS), oT, oD)
                self._neg(u, v, w)
                self._bind_mac_vel(u, v, w)
                self._inc(iT, oT)
                self._inc(iD, oD)
                self._bind("tex_temperature", iT, W, H, D)
                self._bind("tex_density", iD, W, H, D)
                self.launch("adv_sca_mac", g, (BS, BS), oT, oD)
        else:
            raise ValueError(mode)
        self.torch.cuda.synchronize()
        return self.host(oT), self.host(oD)
