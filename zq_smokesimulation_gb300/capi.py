"""ctypes binding of libzqs_gb300.so (include/zqs_capi.h, include/zqs_legacy.h).

The library is the product: this module only loads it and mirrors its C
structs.  Loading fails loudly when the shared object is missing; there is no
fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "lib" / "libzqs_gb300.so"

ZQS_OK, ZQS_EINVAL, ZQS_ENOMEM, ZQS_EUNSUPPORTED, ZQS_ETIMEOUT, ZQS_ECUDA, ZQS_ENOTREADY = range(7)
STATUS_NAMES = {0: "ZQS_OK", 1: "ZQS_EINVAL", 2: "ZQS_ENOMEM", 3: "ZQS_EUNSUPPORTED", 4: "ZQS_ETIMEOUT",
                5: "ZQS_ECUDA", 6: "ZQS_ENOTREADY"}

SOLVER_OPEN, SOLVER_CLOSED, SOLVER_COARSE_OPEN = 0, 1, 2
# ZQ_CUDA_Advection3D.h:7-21 numbering
ADV_VEL_INREG_OUTREG, ADV_VEL_INREG_OUTREG_BFECC, ADV_VEL_INMAC_OUTMAC, ADV_VEL_INMAC_OUTMAC_BFECC, \
    ADV_VEL_INREG_OUTMAC, ADV_VEL_INREG_OUTMAC_BFECC = range(6)
ADV_SCA_MAC, ADV_SCA_MAC_BFECC, ADV_SCA_REG, ADV_SCA_REG_BFECC = range(4)
SOURCE_BOX, SOURCE_SPHERE = 0, 1
MAX_SOURCES = 16

FIELD_U, FIELD_V, FIELD_W, FIELD_TEMPERATURE, FIELD_DENSITY, FIELD_PRESSURE, FIELD_OCCUPANCY, \
    FIELD_DIVERGENCE = range(8)


class Source(C.Structure):
    _fields_ = [("shape", C.c_int32), ("cx", C.c_float), ("cy", C.c_float), ("cz", C.c_float),
                ("hx", C.c_float), ("hy", C.c_float), ("hz", C.c_float), ("density", C.c_float),
                ("temperature", C.c_float)]


class Params(C.Structure):
    _fields_ = [("voxel_size", C.c_float), ("step_time", C.c_float), ("substeps", C.c_int32),
                ("confine", C.c_float), ("buoyancy", C.c_float), ("gravity", C.c_float), ("tamb", C.c_float),
                ("vel_atten", C.c_float), ("temp_atten", C.c_float), ("dens_atten", C.c_float),
                ("solver", C.c_int32), ("sor_iters", C.c_int32), ("omega", C.c_float),
                ("adv_vel_mode", C.c_int32), ("adv_sca_mode", C.c_int32), ("backtrace_full", C.c_int32),
                ("n_sources", C.c_int32), ("sources", Source * MAX_SOURCES), ("sub_size", C.c_int32)]

    def copy(self) -> "Params":
        p = Params()
        C.memmove(C.byref(p), C.byref(self), C.sizeof(Params))
        return p

    def set_sources(self, sources):
        if len(sources) > MAX_SOURCES:
            raise ValueError("at most 16 sources")
        self.n_sources = len(sources)
        for i, s in enumerate(sources):
            self.sources[i] = s


class Object(C.Structure):
    """zqs_object: a voxel mask (host, x fastest) with its size, rotation centre,
    position and velocity in cells per step."""
    _fields_ = [("mask", C.c_void_p), ("size", C.c_int32 * 3), ("center", C.c_int32 * 3), ("pos", C.c_int32 * 3),
                ("vel", C.c_int32 * 3)]


def make_objects(objs):
    """zqs_object array from dicts {mask (sz, sy, sx) bool/uint8, center, pos, vel}; returns (array, keepalive)."""
    arr = (Object * max(1, len(objs)))()
    keep = []
    for q, o in enumerate(objs):
        m = np.ascontiguousarray(o["mask"], dtype=np.uint8)
        keep.append(m)
        arr[q].mask = m.ctypes.data
        sz, sy, sx = m.shape
        arr[q].size[:] = (sx, sy, sz)
        arr[q].center[:] = tuple(int(x) for x in o.get("center", (0, 0, 0)))
        arr[q].pos[:] = tuple(int(x) for x in o["pos"])
        arr[q].vel[:] = tuple(int(x) for x in o.get("vel", (0, 0, 0)))
    return arr, keep


class Camera(C.Structure):
    """zqs_camera: the ray-march view (image size, focal length in pixels,
    row-major inverse view rotation, eye, box, samples per ray, density scale)."""
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("focal", C.c_float), ("inv_view", C.c_float * 9),
                ("eye", C.c_float * 3), ("box_min", C.c_float * 3), ("box_max", C.c_float * 3),
                ("box_size", C.c_float * 3), ("steps", C.c_int32), ("density_scale", C.c_float)]


def default_camera(image_width: int, image_height: int, W: int, H: int, D: int) -> Camera:
    """The viewer's start-up view of a W x H x D volume (zqs_camera_default)."""
    c = Camera()
    load().zqs_camera_default(C.byref(c), image_width, image_height, W, H, D)
    return c


def render_density(density_ptr: int, W: int, H: int, D: int, cam: Camera, rgba_ptr: int, stream: int | None = None):
    """Ray march a dense device density (W*H*D floats, x fastest) into a device
    RGBA image (cam.width * cam.height * 4 floats, bottom row first)."""
    lib = load()
    check(lib.zqs_render_density(C.c_void_p(density_ptr), W, H, D, C.byref(cam), C.c_void_p(rgba_ptr),
                                 C.c_void_p(stream or 0)), "zqs_render_density")


def save_ppm(path, rgba: np.ndarray, background=(0.0, 0.0, 0.0)):
    """Write an RGBA image from the ray march (rows bottom first) as a binary PPM:
    colour + transmittance * background, clamped to [0, 1], top row first."""
    img = np.asarray(rgba, np.float32)
    rgb = img[..., :3] + img[..., 3:4] * np.asarray(background, np.float32)
    rgb = (np.clip(rgb, 0.0, 1.0)[::-1] * 255.0 + 0.5).astype(np.uint8)
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (rgb.shape[1], rgb.shape[0]))
        f.write(rgb.tobytes())


class Stats(C.Structure):
    _fields_ = [("max_abs_div", C.c_double), ("residual_l2", C.c_double), ("div_mean_removed", C.c_double),
                ("free_cells", C.c_int64)]


class SorVariant(C.Structure):
    _fields_ = [("depth", C.c_int32), ("tile_x", C.c_int32), ("tile_y", C.c_int32),
                ("pairs_per_thread", C.c_int32), ("threads", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("smem_bytes", C.c_int64), ("weights_in_registers", C.c_int32), ("registers", C.c_int32),
                ("x_cells_per_thread", C.c_int32), ("split_barrier", C.c_int32)]


class AdjointInfo(C.Structure):
    _fields_ = [("device_bytes", C.c_int64), ("launches_forward", C.c_int64), ("launches_backward", C.c_int64),
                ("nsteps", C.c_int32), ("checkpoint_every", C.c_int32), ("checkpoints", C.c_int32),
                ("pad", C.c_int32)]


class Layout(C.Structure):
    _fields_ = [("W", C.c_int32), ("H", C.c_int32), ("D", C.c_int32), ("pitch_x", C.c_int32),
                ("rows", C.c_int32), ("planes", C.c_int32), ("plane_elems", C.c_int64),
                ("field_elems", C.c_int64)]


# Every symbol include/zqs_capi.h and include/zqs_legacy.h declare with C linkage.
CAPI_SYMBOLS = [
    "zqs_version", "zqs_last_error", "zqs_params_default", "zqs_grid_create", "zqs_grid_destroy",
    "zqs_grid_get_layout", "zqs_grid_set_params", "zqs_grid_get_params", "zqs_grid_upload",
    "zqs_grid_download", "zqs_grid_step", "zqs_grid_use_graph", "zqs_stage_add_force", "zqs_stage_attenuate",
    "zqs_stage_advect_velocity", "zqs_stage_project", "zqs_stage_advect_scalar", "zqs_stage_reinject",
    "zqs_grid_mac_to_regular4", "zqs_grid_stats", "zqs_grid_set_sor_config", "zqs_sor_variant_count",
    "zqs_sor_variant_info", "zqs_grid_set_sor_variant", "zqs_grid_get_sor_choice", "zqs_grid_synchronize",
    "zqs_grid_launch_count",
    "zqs_batch_create", "zqs_batch_destroy", "zqs_batch_step", "zqs_batch_use_graph", "zqs_batch_set_sor_variant",
    "zqs_batch_launch_count", "zqs_batch_synchronize", "zqs_batch_get_sor_choice",
    "zqs_grid_set_force", "zqs_grid_stamp_objects", "zqs_grid_set_coarse_gemm", "zqs_camera_default", "zqs_render_density", "zqs_grid_render",
    "zqs_adjoint_create", "zqs_adjoint_destroy", "zqs_adjoint_forward",
    "zqs_adjoint_backward", "zqs_adjoint_download", "zqs_adjoint_get_info",
    "zqs_debug_inject_tc_stall", "zqs_debug_fail_alloc",
]
LEGACY_C_SYMBOLS = ["ZQ_Cuda_Prepare_Advection", "Advect_Velocity", "Advect_Scalar", "AddForce3D",
                    "Attenuation3D", "zqs_project_sor", "zqs_project_sor_noalloc"]
LEGACY_CXX_SYMBOLS = [
    "_ZN20ZQ_CUDA_MACtoRegular18cu_MAC_to_Regular4EPKfS1_S1_P6float4iii",
    "_ZN20ZQ_CUDA_MACtoRegular18cu_Regular4_to_MACEPK6float4PfS3_S3_iii",
    "_ZN23ZQ_CUDA_PoissonSolver3D40SolveOpenPoissonRedBlackwithOccupy3D_MACEPfS0_S0_PKbiiii",
    "_ZN23ZQ_CUDA_PoissonSolver3D42SolveClosedPoissonRedBlackwithOccupy3D_MACEPfS0_S0_PKbfiiii",
    "_ZN23ZQ_CUDA_PoissonSolver3D21cu_MAC_to_Regular_velEPfS0_S0_PKfS2_S2_iii",
]

_lib = None


class ZQSError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load libzqs_gb300.so (build it with __graft_entry__.build())."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"{p} is missing: build the CUDA library first (python -c 'import "
                                f"__graft_entry__ as g; g.build()')")
    lib = C.CDLL(str(p))
    vp, i, f = C.c_void_p, C.c_int, C.c_float
    lib.zqs_version.restype = i
    lib.zqs_last_error.restype = C.c_char_p
    lib.zqs_params_default.argtypes = [C.POINTER(Params), i, i, i]
    lib.zqs_params_default.restype = None
    lib.zqs_grid_create.argtypes = [C.POINTER(vp), i, i, i]
    lib.zqs_grid_destroy.argtypes = [vp]
    lib.zqs_grid_get_layout.argtypes = [vp, C.POINTER(Layout)]
    lib.zqs_grid_set_params.argtypes = [vp, C.POINTER(Params)]
    lib.zqs_grid_get_params.argtypes = [vp, C.POINTER(Params)]
    lib.zqs_grid_upload.argtypes = [vp, i, vp, i, vp]
    lib.zqs_grid_download.argtypes = [vp, i, vp, i, vp]
    lib.zqs_grid_step.argtypes = [vp, i, vp]
    lib.zqs_grid_use_graph.argtypes = [vp, i]
    lib.zqs_stage_add_force.argtypes = [vp, vp]
    lib.zqs_stage_attenuate.argtypes = [vp, vp]
    lib.zqs_stage_advect_velocity.argtypes = [vp, i, i, vp]
    lib.zqs_stage_project.argtypes = [vp, vp]
    lib.zqs_stage_advect_scalar.argtypes = [vp, i, vp]
    lib.zqs_stage_reinject.argtypes = [vp, vp]
    lib.zqs_grid_mac_to_regular4.argtypes = [vp, vp, i, vp]
    lib.zqs_grid_stats.argtypes = [vp, C.POINTER(Stats), vp]
    lib.zqs_grid_set_sor_config.argtypes = [vp, i, i]
    lib.zqs_grid_launch_count.argtypes = [vp]
    lib.zqs_grid_launch_count.restype = C.c_int64
    lib.zqs_grid_synchronize.argtypes = [vp, vp]
    lib.zqs_sor_variant_count.restype = i
    lib.zqs_sor_variant_info.argtypes = [i, C.POINTER(SorVariant)]
    lib.zqs_grid_set_sor_variant.argtypes = [vp, i, i]
    lib.zqs_debug_inject_tc_stall.argtypes = [i]
    lib.zqs_debug_fail_alloc.argtypes = [i]
    lib.zqs_grid_get_sor_choice.argtypes = [vp, C.POINTER(i), C.POINTER(i), C.POINTER(C.c_float), vp]
    lib.zqs_batch_create.argtypes = [C.POINTER(vp), C.POINTER(vp), i]
    lib.zqs_batch_destroy.argtypes = [vp]
    lib.zqs_batch_step.argtypes = [vp, i, vp]
    lib.zqs_batch_use_graph.argtypes = [vp, i]
    lib.zqs_batch_set_sor_variant.argtypes = [vp, i, i]
    lib.zqs_batch_get_sor_choice.argtypes = [vp, C.POINTER(i), C.POINTER(C.c_float)]
    lib.zqs_batch_launch_count.argtypes = [vp]
    lib.zqs_batch_launch_count.restype = C.c_int64
    lib.zqs_batch_synchronize.argtypes = [vp, vp]
    lib.zqs_grid_set_force.argtypes = [vp, vp, i, vp]
    lib.zqs_grid_stamp_objects.argtypes = [vp, vp, i, i, vp]
    lib.zqs_grid_set_coarse_gemm.argtypes = [vp, i]
    lib.zqs_camera_default.argtypes = [C.POINTER(Camera), i, i, i, i, i]
    lib.zqs_camera_default.restype = None
    lib.zqs_render_density.argtypes = [vp, i, i, i, C.POINTER(Camera), vp, vp]
    lib.zqs_grid_render.argtypes = [vp, C.POINTER(Camera), vp, vp]
    lib.zqs_adjoint_create.argtypes = [C.POINTER(vp), vp, i, i]
    lib.zqs_adjoint_destroy.argtypes = [vp]
    lib.zqs_adjoint_forward.argtypes = [vp, vp, i, vp]
    lib.zqs_adjoint_backward.argtypes = [vp, vp, vp, i, vp]
    lib.zqs_adjoint_download.argtypes = [vp, i, vp, i, vp]
    lib.zqs_adjoint_get_info.argtypes = [vp, C.POINTER(AdjointInfo)]
    # legacy shims
    lib.ZQ_Cuda_Prepare_Advection.argtypes = [C.c_uint, C.c_uint, C.c_uint, f, C.c_uint, f]
    lib.ZQ_Cuda_Prepare_Advection.restype = None
    lib.Advect_Velocity.argtypes = [vp, vp, vp, vp, C.c_bool, i]
    lib.Advect_Velocity.restype = f
    lib.Advect_Scalar.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, i]
    lib.Advect_Scalar.restype = f
    lib.AddForce3D.argtypes = [vp, vp, vp, vp, vp, f, f, f, f, f, i, i, i, i]
    lib.AddForce3D.restype = f
    lib.Attenuation3D.argtypes = [vp, vp, vp, vp, vp, vp, f, f, f, i, i, i]
    lib.Attenuation3D.restype = f
    lib.zqs_project_sor.argtypes = [vp, vp, vp, vp, i, i, i, i, i, f]
    lib.zqs_project_sor.restype = i
    lib.zqs_project_sor_noalloc.argtypes = [vp, vp, vp, vp, i, i, i, i, i, f, vp]
    lib.zqs_project_sor_noalloc.restype = i
    if path is None:
        _lib = lib
    return lib


def last_error() -> str:
    return load().zqs_last_error().decode(errors="replace")


def check(rc: int, what: str = "") -> None:
    if rc != ZQS_OK:
        raise ZQSError(rc, f"{what}: {last_error()}")


def default_params(W: int, H: int, D: int) -> Params:
    p = Params()
    load().zqs_params_default(C.byref(p), W, H, D)
    return p


def sor_variants() -> list[SorVariant]:
    lib = load()
    out = []
    for i in range(lib.zqs_sor_variant_count()):
        v = SorVariant()
        check(lib.zqs_sor_variant_info(i, C.byref(v)), "zqs_sor_variant_info")
        out.append(v)
    return out


def ptr(a: np.ndarray) -> int:
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data


def field_shape(field: int, W: int, H: int, D: int) -> tuple[int, int, int]:
    """numpy shape (z, y, x) of a field in the reference layout."""
    if field == FIELD_U:
        return (D, H, W + 1)
    if field == FIELD_V:
        return (D, H + 1, W)
    if field == FIELD_W:
        return (D + 1, H, W)
    return (D, H, W)


class Grid:
    """One device-resident smoke grid (a zqs_grid handle)."""

    def __init__(self, W: int, H: int, D: int):
        self.lib = load()
        self.W, self.H, self.D = W, H, D
        h = C.c_void_p()
        check(self.lib.zqs_grid_create(C.byref(h), W, H, D), "zqs_grid_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.zqs_grid_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- configuration ---------------------------------------------------------------
    def set_params(self, p: Params):
        check(self.lib.zqs_grid_set_params(self.h, C.byref(p)), "zqs_grid_set_params")

    def params(self) -> Params:
        p = Params()
        check(self.lib.zqs_grid_get_params(self.h, C.byref(p)), "zqs_grid_get_params")
        return p

    def layout(self) -> Layout:
        L = Layout()
        check(self.lib.zqs_grid_get_layout(self.h, C.byref(L)), "zqs_grid_get_layout")
        return L

    def set_sor_config(self, temporal_depth: int = 0, split: bool = False):
        check(self.lib.zqs_grid_set_sor_config(self.h, temporal_depth, 1 if split else 0), "set_sor_config")

    def set_sor_variant(self, index: int = -1, zchunk: int = 0):
        check(self.lib.zqs_grid_set_sor_variant(self.h, index, zchunk), "set_sor_variant")

    def sor_choice(self, stream: int | None = None) -> tuple[int, int, float]:
        """(variant, zchunk, measured us per iteration) the next projection uses."""
        v, z, us = C.c_int(), C.c_int(), C.c_float()
        check(self.lib.zqs_grid_get_sor_choice(self.h, C.byref(v), C.byref(z), C.byref(us),
                                               C.c_void_p(stream) if stream else None), "get_sor_choice")
        return v.value, z.value, us.value

    def use_graph(self, enable: bool):
        check(self.lib.zqs_grid_use_graph(self.h, 1 if enable else 0), "use_graph")

    # -- data -------------------------------------------------------------------------
    def upload(self, field: int, arr: np.ndarray, stream: int | None = None):
        dt = np.uint8 if field == FIELD_OCCUPANCY else np.float32
        shape = field_shape(field, self.W, self.H, self.D)
        a = np.ascontiguousarray(arr, dtype=dt)
        if a.size != int(np.prod(shape)):
            raise ValueError(f"field {field}: expected {shape}, got {arr.shape}")
        check(self.lib.zqs_grid_upload(self.h, field, C.c_void_p(ptr(a)), 0, C.c_void_p(stream or 0)),
              "zqs_grid_upload")
        self._keep = a  # pageable source must outlive the async copy until the next sync
        self.sync(stream)

    def upload_device(self, field: int, dev_ptr: int, stream: int | None = None):
        check(self.lib.zqs_grid_upload(self.h, field, C.c_void_p(dev_ptr), 1, C.c_void_p(stream or 0)),
              "zqs_grid_upload(device)")

    def download(self, field: int, stream: int | None = None) -> np.ndarray:
        dt = np.uint8 if field == FIELD_OCCUPANCY else np.float32
        out = np.empty(field_shape(field, self.W, self.H, self.D), dtype=dt)
        check(self.lib.zqs_grid_download(self.h, field, C.c_void_p(ptr(out)), 0, C.c_void_p(stream or 0)),
              "zqs_grid_download")
        self.sync(stream)
        return out

    def download_into(self, field: int, host_ptr: int, stream: int | None = None):
        check(self.lib.zqs_grid_download(self.h, field, C.c_void_p(host_ptr), 0, C.c_void_p(stream or 0)),
              "zqs_grid_download")

    def upload_from(self, field: int, host_ptr: int, stream: int | None = None):
        check(self.lib.zqs_grid_upload(self.h, field, C.c_void_p(host_ptr), 0, C.c_void_p(stream or 0)),
              "zqs_grid_upload")

    def sync(self, stream: int | None = None):
        check(self.lib.zqs_grid_synchronize(self.h, C.c_void_p(stream or 0)), "zqs_grid_synchronize")

    def load_state(self, occ, u, v, w, T, rho):
        self.upload(FIELD_OCCUPANCY, occ)
        self.upload(FIELD_U, u)
        self.upload(FIELD_V, v)
        self.upload(FIELD_W, w)
        self.upload(FIELD_TEMPERATURE, T)
        self.upload(FIELD_DENSITY, rho)

    def state(self) -> dict:
        return {"u": self.download(FIELD_U), "v": self.download(FIELD_V), "w": self.download(FIELD_W),
                "T": self.download(FIELD_TEMPERATURE), "rho": self.download(FIELD_DENSITY)}

    # -- compute ----------------------------------------------------------------------
    def step(self, n: int = 1, stream: int | None = None):
        check(self.lib.zqs_grid_step(self.h, n, C.c_void_p(stream or 0)), "zqs_grid_step")

    def add_force(self, stream=None):
        check(self.lib.zqs_stage_add_force(self.h, C.c_void_p(stream or 0)), "add_force")

    def attenuate(self, stream=None):
        check(self.lib.zqs_stage_attenuate(self.h, C.c_void_p(stream or 0)), "attenuate")

    def advect_velocity(self, mode: int, is_open: bool = True, stream=None):
        check(self.lib.zqs_stage_advect_velocity(self.h, mode, 1 if is_open else 0, C.c_void_p(stream or 0)),
              "advect_velocity")

    def project(self, stream=None):
        check(self.lib.zqs_stage_project(self.h, C.c_void_p(stream or 0)), "project")

    def advect_scalar(self, mode: int, stream=None):
        check(self.lib.zqs_stage_advect_scalar(self.h, mode, C.c_void_p(stream or 0)), "advect_scalar")

    def reinject(self, stream=None):
        check(self.lib.zqs_stage_reinject(self.h, C.c_void_p(stream or 0)), "reinject")

    def mac_to_regular4(self) -> np.ndarray:
        out = np.empty((self.D, self.H, self.W, 4), dtype=np.float32)
        check(self.lib.zqs_grid_mac_to_regular4(self.h, C.c_void_p(ptr(out)), 0, None), "mac_to_regular4")
        self.sync()
        return out

    def stats(self) -> Stats:
        st = Stats()
        check(self.lib.zqs_grid_stats(self.h, C.byref(st), None), "zqs_grid_stats")
        return st

    def launch_count(self) -> int:
        return int(self.lib.zqs_grid_launch_count(self.h))

    def set_force(self, F: np.ndarray | None):
        """External per-cell force (3, D, H, W) added every step; None removes it."""
        if F is None:
            check(self.lib.zqs_grid_set_force(self.h, None, 0, None), "zqs_grid_set_force")
            return
        a = np.ascontiguousarray(F, dtype=np.float32)
        if a.size != 3 * self.W * self.H * self.D:
            raise ValueError("force must hold 3*W*H*D values")
        check(self.lib.zqs_grid_set_force(self.h, C.c_void_p(ptr(a)), 0, None), "zqs_grid_set_force")
        self.sync()

    def stamp_objects(self, objs, closed_walls: int = 0, stream=None):
        """Moving voxel objects (zqs_grid_stamp_objects); objs as for make_objects;
        closed_walls 0 none, 1 (or True) all six walls, 2 all but the y = H-1 layer."""
        arr, keep = make_objects(objs)
        check(self.lib.zqs_grid_stamp_objects(self.h, C.cast(arr, C.c_void_p), len(objs), int(closed_walls),
                                              C.c_void_p(stream or 0)), "zqs_grid_stamp_objects")
        del keep

    def set_coarse_gemm(self, mode: int):
        """Coarse solver's obstacle-free blocks: 1 tensor cores (3xTF32), 0 FP32 SIMT (exact)."""
        check(self.lib.zqs_grid_set_coarse_gemm(self.h, int(mode)), "zqs_grid_set_coarse_gemm")

    def render(self, cam: Camera, rgba_ptr: int, stream: int | None = None):
        """Ray march the current density into a device RGBA image (zqs_grid_render)."""
        check(self.lib.zqs_grid_render(self.h, C.byref(cam), C.c_void_p(rgba_ptr), C.c_void_p(stream or 0)),
              "zqs_grid_render")

    def set_force_device(self, dev_ptr: int, stream: int | None = None):
        check(self.lib.zqs_grid_set_force(self.h, C.c_void_p(dev_ptr), 1, C.c_void_p(stream or 0)),
              "zqs_grid_set_force")


class Batch:
    """Many grids advanced together (a zqs_batch handle): one persistent launch
    per stage over all members' tiles, replayed as a CUDA graph.  The members
    stay usable as Grid objects; after step() call sync() (or pass the stream
    the members are read on) before downloading them."""

    def __init__(self, grids: list[Grid]):
        self.lib = load()
        self.grids = list(grids)  # the handles must outlive the batch
        arr = (C.c_void_p * len(self.grids))(*[g.h.value for g in self.grids])
        h = C.c_void_p()
        check(self.lib.zqs_batch_create(C.byref(h), arr, len(self.grids)), "zqs_batch_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.zqs_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def step(self, n: int = 1, stream: int | None = None):
        check(self.lib.zqs_batch_step(self.h, n, C.c_void_p(stream or 0)), "zqs_batch_step")

    def use_graph(self, enable: bool):
        check(self.lib.zqs_batch_use_graph(self.h, 1 if enable else 0), "zqs_batch_use_graph")

    def set_sor_variant(self, index: int = -1, zchunk: int = 0):
        check(self.lib.zqs_batch_set_sor_variant(self.h, index, zchunk), "zqs_batch_set_sor_variant")

    def sync(self, stream: int | None = None):
        check(self.lib.zqs_batch_synchronize(self.h, C.c_void_p(stream or 0)), "zqs_batch_synchronize")

    def launch_count(self) -> int:
        return int(self.lib.zqs_batch_launch_count(self.h))

    def sor_choice(self) -> tuple[int, float]:
        """(variant, measured us per iteration) of the batched SOR passes."""
        v, us = C.c_int(), C.c_float()
        check(self.lib.zqs_batch_get_sor_choice(self.h, C.byref(v), C.byref(us)), "batch sor_choice")
        return v.value, us.value


class Adjoint:
    """Reverse-mode session (a zqs_adjoint handle) over nsteps steps of a grid
    with a control force, for losses on the final density."""

    def __init__(self, grid: Grid, nsteps: int, checkpoint_every: int = 8):
        self.lib = load()
        self.grid = grid
        self.nsteps = nsteps
        h = C.c_void_p()
        check(self.lib.zqs_adjoint_create(C.byref(h), grid.h, nsteps, checkpoint_every), "zqs_adjoint_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.zqs_adjoint_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, F: np.ndarray | None):
        g = self.grid
        if F is None:
            check(self.lib.zqs_adjoint_forward(self.h, None, 0, None), "zqs_adjoint_forward")
        else:
            a = np.ascontiguousarray(F, dtype=np.float32)
            check(self.lib.zqs_adjoint_forward(self.h, C.c_void_p(ptr(a)), 0, None), "zqs_adjoint_forward")
        g.sync()

    def forward_device(self, dev_ptr: int, stream: int | None = None):
        check(self.lib.zqs_adjoint_forward(self.h, C.c_void_p(dev_ptr), 1, C.c_void_p(stream or 0)),
              "zqs_adjoint_forward")

    def backward(self, g_density: np.ndarray) -> np.ndarray:
        g = self.grid
        gd = np.ascontiguousarray(g_density, dtype=np.float32)
        out = np.empty((3, g.D, g.H, g.W), np.float32)
        check(self.lib.zqs_adjoint_backward(self.h, C.c_void_p(ptr(gd)), C.c_void_p(ptr(out)), 0, None),
              "zqs_adjoint_backward")
        g.sync()
        return out

    def backward_device(self, g_density_ptr: int, grad_ptr: int, stream: int | None = None):
        check(self.lib.zqs_adjoint_backward(self.h, C.c_void_p(g_density_ptr), C.c_void_p(grad_ptr), 1,
                                            C.c_void_p(stream or 0)), "zqs_adjoint_backward")

    def initial_adjoint(self, field: int) -> np.ndarray:
        g = self.grid
        out = np.empty(field_shape(field, g.W, g.H, g.D), np.float32)
        check(self.lib.zqs_adjoint_download(self.h, field, C.c_void_p(ptr(out)), 0, None), "zqs_adjoint_download")
        g.sync()
        return out

    def info(self) -> AdjointInfo:
        inf = AdjointInfo()
        check(self.lib.zqs_adjoint_get_info(self.h, C.byref(inf)), "zqs_adjoint_get_info")
        return inf
