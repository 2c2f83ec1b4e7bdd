"""GPU parity: the CUDA library (through its C ABI) against the FP32 CPU oracle.

The kernels reproduce the oracle's operation order with no contraction, so
FP32 results are expected to be bit-identical (-0 == +0); the floating-point
tolerances of the path (relative L2 1e-5 per step, 1e-4 after 100 steps) are
asserted as well where a trajectory is compared.
"""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_l2
from zq_smokesimulation_gb300 import capi
from zq_smokesimulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

FIELDS = ("u", "v", "w", "T", "rho")
TOL_STEP = 1e-5
TOL_100 = 1e-4


def gpu_grid(w, sor=(2, False), graph=True):
    g = capi.Grid(w.W, w.H, w.D)
    g.set_params(w.params)
    g.set_sor_config(*sor)
    g.use_graph(graph)
    g.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
    return g


def assert_same(gpu: dict, ref: dict, keys=FIELDS, what=""):
    for k in keys:
        a, b = gpu[k], ref[k]
        assert a.shape == b.shape, (what, k)
        if not np.array_equal(a, b):
            bad = np.argwhere(a != b)
            raise AssertionError(f"{what} {k}: {len(bad)} mismatches, first {bad[:3].tolist()}, "
                                 f"gpu {a[tuple(bad[0])]!r} oracle {b[tuple(bad[0])]!r}, "
                                 f"relL2 {rel_l2(a, b):.3e}")


SMALL = [(9, 11, 7), (16, 12, 10), (5, 7, 3), (33, 17, 9)]


@pytest.mark.parametrize("dims", SMALL)
def test_stage_add_force(zqs_lib, oracle32, dims):
    w = wl.small_case(*dims, vel_amp=0.3)
    w.params.confine = 2.5
    g = gpu_grid(w)
    g.add_force()
    st = oracle32.state(w)
    oracle32.add_force(w.W, w.H, w.D, st, w.occ, w.params)
    assert_same(g.state(), st, what="add_force")


@pytest.mark.parametrize("dims", SMALL[:2])
def test_stage_attenuate(zqs_lib, oracle32, dims):
    w = wl.small_case(*dims)
    w.params.vel_atten, w.params.temp_atten, w.params.dens_atten = 0.97, 0.93, 0.91
    g = gpu_grid(w)
    g.attenuate()
    st = oracle32.state(w)
    oracle32.attenuate(w.W, w.H, w.D, st, w.occ, w.params)
    assert_same(g.state(), st, what="attenuate")


VEL_MODES = [capi.ADV_VEL_INMAC_OUTMAC, capi.ADV_VEL_INREG_OUTMAC, capi.ADV_VEL_INREG_OUTREG,
             capi.ADV_VEL_INMAC_OUTMAC_BFECC, capi.ADV_VEL_INREG_OUTMAC_BFECC, capi.ADV_VEL_INREG_OUTREG_BFECC]


@pytest.mark.parametrize("mode", VEL_MODES)
@pytest.mark.parametrize("is_open", [True, False])
@pytest.mark.parametrize("dims", SMALL[:3])
def test_stage_advect_velocity(zqs_lib, oracle32, mode, is_open, dims):
    w = wl.small_case(*dims, vel_amp=0.4, substeps=5)
    w.params.step_time = 0.3
    g = gpu_grid(w)
    g.advect_velocity(mode, is_open)
    st = oracle32.state(w)
    assert oracle32.advect_velocity(w.W, w.H, w.D, st, w.occ, w.params, mode, is_open) == 0
    assert_same(g.state(), st, keys=("u", "v", "w"), what=f"advect_velocity mode {mode}")


@pytest.mark.parametrize("mode", [capi.ADV_SCA_MAC, capi.ADV_SCA_REG, capi.ADV_SCA_MAC_BFECC, capi.ADV_SCA_REG_BFECC])
@pytest.mark.parametrize("full", [0, 1])
@pytest.mark.parametrize("dims", SMALL[:3])
def test_stage_advect_scalar(zqs_lib, oracle32, mode, full, dims):
    w = wl.small_case(*dims, vel_amp=0.4, substeps=3)
    w.params.step_time = 0.3
    w.params.backtrace_full = full
    g = gpu_grid(w)
    g.advect_scalar(mode)
    st = oracle32.state(w)
    assert oracle32.advect_scalar(w.W, w.H, w.D, st, w.occ, w.params, mode) == 0
    assert_same(g.state(), st, keys=("T", "rho"), what=f"advect_scalar mode {mode}")


def test_stage_reinject(zqs_lib, oracle32):
    w = wl.small_case(16, 12, 10)
    g = gpu_grid(w)
    g.reinject()
    st = oracle32.state(w)
    oracle32.reinject(w.W, w.H, w.D, st, w.params)
    assert_same(g.state(), st, keys=("T", "rho"), what="reinject")


@pytest.mark.parametrize("closed", [False, True])
@pytest.mark.parametrize("sor", [(1, True), (1, False), (2, False), (3, False), (4, False)])
@pytest.mark.parametrize("dims,K", [((9, 11, 7), 7), ((33, 17, 40), 9), ((64, 20, 13), 4)])
def test_stage_project(zqs_lib, oracle32, closed, sor, dims, K):
    w = wl.small_case(*dims, closed=closed, K=K, vel_amp=0.3)
    g = gpu_grid(w, sor=sor)
    g.project()
    st = oracle32.state(w)
    pr, div, stats = oracle32.project(w.W, w.H, w.D, st, w.occ, w.params, want=True)
    out = g.state()
    out["p"] = g.download(capi.FIELD_PRESSURE)
    out["div"] = g.download(capi.FIELD_DIVERGENCE) * (w.occ == 0)
    st["p"], st["div"] = pr, div
    assert_same(out, st, keys=("u", "v", "w", "p", "div"), what=f"project sor={sor}")
    gs = g.stats()
    assert gs.free_cells == stats.free_cells
    assert gs.max_abs_div == pytest.approx(stats.max_abs_div, rel=1e-12, abs=1e-30)
    assert gs.residual_l2 == pytest.approx(stats.residual_l2, rel=1e-9)
    if closed:
        assert gs.div_mean_removed == stats.div_mean_removed


def test_mac_to_regular4(zqs_lib, oracle32):
    w = wl.small_case(13, 9, 6, vel_amp=1.0)
    g = gpu_grid(w)
    c4 = g.mac_to_regular4()
    ref = oracle32.mac_to_regular4(w.W, w.H, w.D, oracle32.arr(w.u), oracle32.arr(w.v), oracle32.arr(w.w))
    assert np.array_equal(c4, ref)


COMBOS = [(capi.ADV_VEL_INMAC_OUTMAC, capi.ADV_SCA_MAC), (capi.ADV_VEL_INREG_OUTREG, capi.ADV_SCA_REG),
          (capi.ADV_VEL_INREG_OUTMAC, capi.ADV_SCA_MAC),
          (capi.ADV_VEL_INMAC_OUTMAC_BFECC, capi.ADV_SCA_MAC_BFECC),
          (capi.ADV_VEL_INREG_OUTREG_BFECC, capi.ADV_SCA_REG_BFECC),
          (capi.ADV_VEL_INREG_OUTMAC_BFECC, capi.ADV_SCA_MAC)]


@pytest.mark.parametrize("vm,sm", COMBOS)
@pytest.mark.parametrize("closed", [False, True])
@pytest.mark.parametrize("graph", [True, False])
def test_full_steps(zqs_lib, oracle32, vm, sm, closed, graph):
    w = wl.small_case(17, 14, 11, closed=closed, K=13, substeps=4, vel_mode=vm, sca_mode=sm, vel_amp=0.2)
    w.params.step_time = 0.2
    g = gpu_grid(w, graph=graph)
    g.step(4)
    st = oracle32.state(w)
    rc, _ = oracle32.step(w.W, w.H, w.D, st, w.occ, w.params, 4)
    assert rc == 0
    out = g.state()
    for k in FIELDS:
        assert rel_l2(out[k], st[k]) <= TOL_STEP, k
    assert_same(out, st, what=f"4 steps vm={vm} sm={sm} closed={closed} graph={graph}")


def test_golden_fixtures_gpu(zqs_lib):
    gdir = Path(__file__).parent / "golden"
    for f in sorted(gdir.glob("*.npz")):
        gd = np.load(f)
        meta = json.loads(str(gd["meta"]))
        w = wl.small_case(*meta["dims"], seed=meta["seed"], K=meta["K"], substeps=meta["substeps"],
                          closed=meta["closed"], vel_mode=meta["vel_mode"], sca_mode=meta["sca_mode"])
        g = gpu_grid(w)
        g.step(meta["steps"])
        out = g.state()
        assert_same(out, {k: gd[f"f32_{k}"] for k in FIELDS}, what=f.name)
        for k in FIELDS:   # and the FP64 oracle's error bound
            assert rel_l2(out[k], gd[f"f64_{k}"]) < 1e-5, (f.name, k)


def _trajectory(w, oracle32, oracle64, checkpoints, tag):
    """Steps the GPU grid, the FP32 oracle and the FP64 oracle of workload w to
    each checkpoint; asserts the GPU against the FP32 oracle (relative L2 1e-5
    after the first step, 1e-4 later, and bit for bit) and returns the
    relative L2 errors of the GPU and of the FP32 oracle against FP64."""
    g = gpu_grid(w)
    s32, s64 = oracle32.state(w), oracle64.state(w)
    done, rows = 0, []
    for n in checkpoints:
        g.step(n - done)
        for o, s in ((oracle32, s32), (oracle64, s64)):
            rc, _ = o.step(w.W, w.H, w.D, s, w.occ, w.params, n - done)
            assert rc == 0
        done = n
        out = g.state()
        tol = TOL_STEP if n == 1 else TOL_100
        for k in FIELDS:
            e = rel_l2(out[k], s32[k])
            assert e <= tol, (tag, n, k, e)
        assert_same(out, s32, what=f"{tag} step {n}")
        row = {"step": n}
        for k in FIELDS:
            row[k] = (rel_l2(out[k], s64[k]), rel_l2(s32[k], s64[k]))
            assert np.isfinite(row[k][0]) and row[k][0] == row[k][1], (tag, n, k)
        rows.append(row)
        print(f"{tag} step {n}: relL2 vs FP64 (GPU = FP32 oracle): " +
              ", ".join(f"{k} {row[k][0]:.2e}" for k in FIELDS))
    g.close()
    return rows, out


def test_plain64_100_steps(zqs_lib, oracle32, oracle64):
    """Configuration 0 (64^3, closed walls with an open top, sphere source,
    K=200, omega 1.9) for 100 steps: the GPU against the FP32 oracle at steps
    1 and 100, and the error of both against the FP64 oracle."""
    rows, out = _trajectory(wl.make("plain64"), oracle32, oracle64, (1, 100), "plain64")
    assert float(out["rho"].sum()) > 100.0   # smoke has risen and spread
    # one step from the seeded state stays close to FP64; a hundred steps of
    # the buoyant plume amplify rounding differences (the flow is unstable)
    assert max(rows[0][k][0] for k in FIELDS) < 1e-4


def test_plain128_obstacle_trajectory(zqs_lib, oracle32, oracle64):
    """Configuration 1 (128^3, the box obstacle [48,80]x[56,72]x[48,80],
    sphere source r=10 at (64,12,64), K=400, omega 1.9): GPU against the FP32
    oracle at steps 1 and 100, both against FP64."""
    w = wl.make("plain128_obs")
    assert w.params.sor_iters == 400 and int(w.occ[60, 60, 60]) == 1
    rows, out = _trajectory(w, oracle32, oracle64, (1, 100), "plain128_obs")
    assert max(rows[0][k][0] for k in FIELDS) < 1e-4
    lu, lv, lw = wl.live_faces(w.occ)
    assert np.all(out["u"][~lu] == 0) and np.all(out["v"][~lv] == 0) and np.all(out["w"][~lw] == 0)


@pytest.mark.long
def test_plain128_obstacle_500_steps(zqs_lib, oracle32, oracle64):
    """Configuration 1 to step 500 (checkpoints 1, 100, 500); several minutes
    of oracle time, so it runs with --runlong."""
    _trajectory(wl.make("plain128_obs"), oracle32, oracle64, (1, 100, 500), "plain128_obs")


def test_plain512_one_step_vs_oracle(zqs_lib, oracle32):
    """Configuration 2 at 512^3 (four seeded sphere sources) for one step at
    K=4: every field bit for bit against the FP32 oracle."""
    w = wl.make("plain512", K=4)
    g = gpu_grid(w)
    g.step(1)
    out = g.state()
    g.close()
    st = oracle32.state(w)
    rc, _ = oracle32.step(w.W, w.H, w.D, st, w.occ, w.params, 1)
    assert rc == 0
    for k in FIELDS:
        assert rel_l2(out[k], st[k]) <= TOL_STEP, k
    assert_same(out, st, what="plain512 step")


def _variants():
    from zq_smokesimulation_gb300 import capi as c
    try:
        return list(range(len(c.sor_variants())))
    except Exception:
        return list(range(10))


@pytest.mark.parametrize("variant", _variants())
@pytest.mark.parametrize("case", ["plain256", "odd"])
def test_sor_fused_variants_equal_split(zqs_lib, variant, case):
    """Colour-race self-check: every temporally blocked SOR variant reproduces
    one-colour-per-launch sweeps bit for bit (K=11 also exercises the
    shorter remainder pass), at full size and on an odd-sized obstacle grid."""
    if case == "plain256":
        w = wl.make("plain256", K=11)
    else:
        w = wl.small_case(37, 29, 23, K=11, vel_amp=0.3)
    info = capi.sor_variants()[variant]
    if info.ctas_per_sm < 1:
        pytest.skip("variant does not fit this device")
    g1 = gpu_grid(w, sor=(1, True))
    g1.project()
    g2 = gpu_grid(w, sor=(info.depth, False))
    for zchunk in (0, 5):
        g2.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
        g2.set_sor_variant(variant, zchunk)
        g2.project()
        g2.sync()   # raises on a device-side wait that gave up (split-barrier variants)
        a = {k: g1.download(f) for k, f in (("p", capi.FIELD_PRESSURE), ("v", capi.FIELD_V))}
        b = {k: g2.download(f) for k, f in (("p", capi.FIELD_PRESSURE), ("v", capi.FIELD_V))}
        assert_same(b, a, keys=("p", "v"), what=f"variant {variant} zchunk {zchunk}")


@pytest.mark.parametrize("shape", [(160, 96, 120), (96, 96, 300), (128, 256, 128)])
@pytest.mark.parametrize("depth", [1, 2])
def test_sor_default_partition_equal_split(zqs_lib, shape, depth):
    """The default fused pass with its automatic z chunk reproduces one-colour
    sweeps bit for bit on grids whose tiles and z chunks are ragged, with an
    obstacle; K=5 also runs the depth-1 remainder pass."""
    w = wl.small_case(*shape, K=5, vel_amp=0.3)
    g1 = gpu_grid(w, sor=(1, True))
    g1.project()
    g2 = gpu_grid(w, sor=(depth, False))
    g2.project()
    a = {k: g1.download(f) for k, f in (("p", capi.FIELD_PRESSURE), ("v", capi.FIELD_V))}
    b = {k: g2.download(f) for k, f in (("p", capi.FIELD_PRESSURE), ("v", capi.FIELD_V))}
    assert_same(b, a, keys=("p", "v"), what=f"{shape} depth {depth}")


def test_plain256_one_step_vs_oracle(zqs_lib, oracle32):
    w = wl.make("plain256", K=8)
    g = gpu_grid(w)
    g.step(1)
    st = oracle32.state(w)
    oracle32.step(w.W, w.H, w.D, st, w.occ, w.params, 1)
    out = g.state()
    for k in FIELDS:
        assert rel_l2(out[k], st[k]) <= TOL_STEP, k
    assert_same(out, st, what="plain256 step")


def test_projection_converges_at_256(zqs_lib):
    """Size-independent property: more SOR iterations never raise max|div|."""
    w = wl.make("plain256", K=1)
    w.u, w.v, w.w = wl.initial_velocity(w.occ, 3, amp=1.0)
    res = []
    for K in (10, 100, 600):
        w.params.sor_iters = K
        g = gpu_grid(w)
        g.project()
        res.append(g.stats().residual_l2)
        g.close()
    assert res[0] > res[1] > res[2]


def test_step_is_deterministic(zqs_lib):
    w = wl.make("plain128_obs", K=40)
    outs = []
    for _ in range(2):
        g = gpu_grid(w)
        g.step(3)
        outs.append(g.state())
        g.close()
    assert_same(outs[0], outs[1], what="repeat")


def test_obstacle_faces_stay_zero(zqs_lib):
    w = wl.make("plain128_obs", K=40)
    g = gpu_grid(w)
    g.step(5)
    out = g.state()
    lu, lv, lw = wl.live_faces(w.occ)
    assert np.all(out["u"][~lu] == 0) and np.all(out["v"][~lv] == 0) and np.all(out["w"][~lw] == 0)
    assert np.isfinite(out["rho"]).all() and np.abs(out["v"]).max() > 0


# ---------------------------------------------------------------- legacy shims

def _legacy_state(w):
    return {k: np.ascontiguousarray(getattr(w, k), np.float32).copy() for k in FIELDS}


def test_legacy_advect_velocity_and_scalar(zqs_lib, oracle32):
    w = wl.small_case(12, 10, 9, vel_amp=0.4, substeps=3)
    lib = zqs_lib
    h = float(w.params.voxel_size)
    dt_sub = np.float32(np.float32(0.3) / np.float32(3))
    w.params.step_time = 0.3
    lib.ZQ_Cuda_Prepare_Advection(w.W, w.H, w.D, h, 3, float(dt_sub))
    st = _legacy_state(w)
    occ = np.ascontiguousarray(w.occ, np.uint8)
    ms = lib.Advect_Velocity(st["u"].ctypes.data, st["v"].ctypes.data, st["w"].ctypes.data, occ.ctypes.data, True,
                             capi.ADV_VEL_INMAC_OUTMAC)
    assert ms >= 0, capi.last_error()
    ref = oracle32.state(w)
    oracle32.advect_velocity(w.W, w.H, w.D, ref, w.occ, w.params, capi.ADV_VEL_INMAC_OUTMAC, True)
    assert_same(st, ref, keys=("u", "v", "w"), what="Advect_Velocity")
    outT = np.empty_like(st["T"])
    outD = np.empty_like(st["rho"])
    ms = lib.Advect_Scalar(st["u"].ctypes.data, st["v"].ctypes.data, st["w"].ctypes.data, occ.ctypes.data,
                           st["T"].ctypes.data, st["rho"].ctypes.data, outT.ctypes.data, outD.ctypes.data,
                           capi.ADV_SCA_REG)
    assert ms >= 0, capi.last_error()
    oracle32.advect_scalar(w.W, w.H, w.D, ref, w.occ, w.params, capi.ADV_SCA_REG)
    assert np.array_equal(outT, ref["T"]) and np.array_equal(outD, ref["rho"])
    # BFECC through the same entry points (the reference's Advect_Scalar
    # returns zeros for these types; here the three passes run)
    ms = lib.Advect_Velocity(st["u"].ctypes.data, st["v"].ctypes.data, st["w"].ctypes.data, occ.ctypes.data, False,
                             capi.ADV_VEL_INMAC_OUTMAC_BFECC)
    assert ms >= 0, capi.last_error()
    oracle32.advect_velocity(w.W, w.H, w.D, ref, w.occ, w.params, capi.ADV_VEL_INMAC_OUTMAC_BFECC, False)
    assert_same(st, ref, keys=("u", "v", "w"), what="Advect_Velocity BFECC")
    ms = lib.Advect_Scalar(st["u"].ctypes.data, st["v"].ctypes.data, st["w"].ctypes.data, occ.ctypes.data,
                           st["T"].ctypes.data, st["rho"].ctypes.data, outT.ctypes.data, outD.ctypes.data,
                           capi.ADV_SCA_MAC_BFECC)
    assert ms >= 0, capi.last_error()
    ref["T"], ref["rho"] = st["T"].copy(), st["rho"].copy()   # the inputs (the REG call above wrote ref's)
    oracle32.advect_scalar(w.W, w.H, w.D, ref, w.occ, w.params, capi.ADV_SCA_MAC_BFECC)
    assert np.array_equal(outT, ref["T"]) and np.array_equal(outD, ref["rho"])
    assert float(np.abs(outD).sum()) > 0.0
    # an unknown type is refused and leaves the arrays untouched
    before = st["u"].copy()
    ms = lib.Advect_Velocity(st["u"].ctypes.data, st["v"].ctypes.data, st["w"].ctypes.data, occ.ctypes.data, True,
                             6)
    assert ms == -capi.ZQS_EINVAL and np.array_equal(st["u"], before)


def test_legacy_addforce_attenuation_projection(zqs_lib, oracle32):
    w = wl.small_case(14, 11, 9, vel_amp=0.3, K=15)
    w.params.gravity = 0.0  # the reference AddForce3D has no density term
    lib = zqs_lib
    st = _legacy_state(w)
    occ = np.ascontiguousarray(w.occ, np.uint8)
    p = w.params
    ms = lib.AddForce3D(st["u"].ctypes.data, st["v"].ctypes.data, st["w"].ctypes.data, occ.ctypes.data,
                        st["T"].ctypes.data, float(p.voxel_size), float(p.step_time), float(p.buoyancy),
                        float(p.confine), float(p.tamb), w.W, w.H, w.D, 0)
    assert ms >= 0, capi.last_error()
    ref = oracle32.state(w)
    oracle32.add_force(w.W, w.H, w.D, ref, w.occ, p)
    assert_same(st, ref, keys=("u", "v", "w"), what="AddForce3D")
    ms = lib.Attenuation3D(st["u"].ctypes.data, st["v"].ctypes.data, st["w"].ctypes.data, st["T"].ctypes.data,
                           st["rho"].ctypes.data, occ.ctypes.data, 0.9, 0.8, 0.7, w.W, w.H, w.D)
    assert ms >= 0
    p.vel_atten, p.temp_atten, p.dens_atten = 0.9, 0.8, 0.7
    oracle32.attenuate(w.W, w.H, w.D, ref, w.occ, p)
    assert_same(st, ref, what="Attenuation3D")
    rc = lib.zqs_project_sor(st["u"].ctypes.data, st["v"].ctypes.data, st["w"].ctypes.data, occ.ctypes.data, w.W,
                             w.H, w.D, capi.SOLVER_OPEN, 15, C.c_float(1.9))
    assert rc == 0, capi.last_error()
    oracle32.project(w.W, w.H, w.D, ref, w.occ, p)
    assert_same(st, ref, keys=("u", "v", "w"), what="zqs_project_sor")


# ---------------------------------------------------------------- edge cases

def test_tiny_and_degenerate_grids(zqs_lib, oracle32):
    for dims in ((2, 2, 2), (3, 2, 5), (2, 9, 3)):
        w = wl.small_case(*dims, obstacle=False, K=3, substeps=2)
        w.occ[:] = 0
        g = gpu_grid(w)
        g.step(2)
        st = oracle32.state(w)
        oracle32.step(w.W, w.H, w.D, st, w.occ, w.params, 2)
        assert_same(g.state(), st, what=f"tiny {dims}")
    # every cell occupied: nothing moves, nothing faults
    w = wl.small_case(6, 5, 4, K=3)
    w.occ[:] = 1
    g = gpu_grid(w)
    g.step(2)
    st = oracle32.state(w)
    oracle32.step(w.W, w.H, w.D, st, w.occ, w.params, 2)
    assert_same(g.state(), st, what="all occupied")


def test_non_power_of_two_voxel_size(zqs_lib, oracle32):
    w = wl.small_case(12, 10, 8, vel_amp=0.3)
    w.params.voxel_size = 1.0 / 12.0   # not a power of two: the division path
    g = gpu_grid(w)
    g.step(2)
    st = oracle32.state(w)
    oracle32.step(w.W, w.H, w.D, st, w.occ, w.params, 2)
    assert_same(g.state(), st, what="h=1/12")


def test_no_sources_and_nan_input(zqs_lib, oracle32):
    w = wl.small_case(10, 9, 8)
    w.params.n_sources = 0
    w.T[3, 3, 3] = np.nan
    g = gpu_grid(w)
    g.step(1)
    out = g.state()
    st = oracle32.state(w)
    oracle32.step(w.W, w.H, w.D, st, w.occ, w.params, 1)
    for k in FIELDS:
        assert np.array_equal(np.isnan(out[k]), np.isnan(st[k])), k
        m = ~np.isnan(st[k])
        assert np.array_equal(out[k][m], st[k][m]), k


def test_errors_are_reported(zqs_lib):
    h = C.c_void_p()
    assert zqs_lib.zqs_grid_create(C.byref(h), 1, 4, 4) == capi.ZQS_EINVAL
    assert "dimension" in capi.last_error()
    g = capi.Grid(4, 4, 4)
    with pytest.raises(capi.ZQSError) as e:
        g.step(1)
    assert e.value.code == capi.ZQS_ENOTREADY
    p = wl.smoke_params(4, 3)
    p.substeps = 0
    with pytest.raises(capi.ZQSError) as e:
        g.set_params(p)
    assert e.value.code == capi.ZQS_EINVAL
    p.substeps = 2
    p.adv_vel_mode = 6
    with pytest.raises(capi.ZQSError) as e:
        g.set_params(p)
    assert e.value.code == capi.ZQS_EINVAL
    p.adv_vel_mode = capi.ADV_VEL_INMAC_OUTMAC_BFECC
    g.set_params(p)
    g.upload(capi.FIELD_OCCUPANCY, np.zeros((4, 4, 4), np.uint8))
    g.step(1)
    with pytest.raises(capi.ZQSError):
        g.set_sor_config(9)
    g.close()
