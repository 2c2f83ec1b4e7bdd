"""The C++ host API with the reference's class names (include/zqs_smoke3d.h).

A small driver (tests/cpp/smoke3d_driver.cpp) is compiled against the built
library.  CPU: config parsing (the reference's key/value format plus the added
keys) and ZQ_InitFineGrid3D against the Python workload builders.  GPU: the
resident path (ZQ_SmokeSimulation3D::Init + Run, .di3 frames) equals the
free-function path (ZQ_UpdateOneFrame3D) and the FP32 oracle bit for bit.
"""
import ctypes as C
import math
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from conftest import rel_l2
from zq_smokesimulation_gb300 import capi
from zq_smokesimulation_gb300 import workloads as wl

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def driver(zqs_lib, tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ missing")
    out = tmp_path_factory.mktemp("drv") / "smoke3d_driver"
    libdir = ROOT / "zq_smokesimulation_gb300" / "lib"
    cmd = [gxx, "-std=c++17", "-O1", f"-I{ROOT / 'include'}", str(ROOT / "tests" / "cpp" / "smoke3d_driver.cpp"),
           f"-L{libdir}", "-lzqs_gb300", f"-Wl,-rpath,{libdir}", "-o", str(out)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return out


CONFIG = """resolution 24 20 16
subSize 4
source 0.5 0.15 0.5 0.1 0.08 0.12 1.0 1.0
sphereSource 0.3 0.2 0.6 0.12 0.7 0.5
Tamb 0
confineCoeff 0.2
steps 4
stepTime 0.05
frameCount 3
maxIter 12
omega 1.9
alpha 0.1
beta 0.5
velAttenFactor 0.99
tempAttenCoeff 0.2
densityAttenFactor 0.99
wallsExceptTop true
obstacleBox 8 10 9 11 5 8
noiseAmp 0.05
seed 3
advVelType inMAC_outMAC
advScaType MAC
globalGridSolver TOTAL_CLOSED_POISSON_SOR
"""


def run_driver(driver, mode, cfg_text, outdir):
    outdir.mkdir(parents=True, exist_ok=True)
    cfg = outdir / "config.txt"
    cfg.write_text(cfg_text)
    r = subprocess.run([str(driver), mode, str(cfg), str(outdir)], capture_output=True, text=True)
    assert r.returncode == 0, (mode, r.returncode, r.stdout, r.stderr)
    return outdir


def load_setup(outdir, W, H, D):
    p = capi.Params.from_buffer_copy((outdir / "params.bin").read_bytes())
    occ = np.fromfile(outdir / "occupancy.bin", np.uint8).reshape(D, H, W)
    st = load_guide(outdir / "init.guidedat", W, H, D)
    return p, occ, st


def load_guide(path, W, H, D):
    a = np.fromfile(path, np.float32)
    nu, nv, nw, n = (W + 1) * H * D, W * (H + 1) * D, W * H * (D + 1), W * H * D
    assert a.size == nu + nv + nw + 2 * n
    o = np.cumsum([0, nu, nv, nw, n, n])
    return {"u": a[o[0]:o[1]].reshape(D, H, W + 1), "v": a[o[1]:o[2]].reshape(D, H + 1, W),
            "w": a[o[2]:o[3]].reshape(D + 1, H, W), "rho": a[o[3]:o[4]].reshape(D, H, W),
            "T": a[o[4]:o[5]].reshape(D, H, W)}


def load_di3(path):
    b = Path(path).read_bytes()
    assert b[:5] == b"float" and len(b) >= 33
    W, H, D, ch = np.frombuffer(b[16:32], np.int32)
    assert ch == 1
    return np.frombuffer(b[33:], np.float32).reshape(D, H, W)


def test_config_and_initial_state(driver, tmp_path):
    out = run_driver(driver, "parse", CONFIG, tmp_path / "p")
    W, H, D = 24, 20, 16
    p, occ, st = load_setup(out, W, H, D)
    assert (p.substeps, p.sor_iters, p.solver) == (4, 12, capi.SOLVER_OPEN)  # wallsExceptTop -> open solver
    assert p.voxel_size == np.float32(1.0 / 24) and p.omega == np.float32(1.9)
    assert p.gravity == np.float32(0.1) and p.buoyancy == np.float32(0.5) and p.confine == np.float32(0.2)
    assert p.vel_atten == np.float32(0.99) and p.dens_atten == np.float32(0.99)
    assert p.temp_atten == np.float32(math.exp(np.float32(-0.05) * np.float32(0.2)))
    assert (p.adv_vel_mode, p.adv_sca_mode) == (capi.ADV_VEL_INMAC_OUTMAC, capi.ADV_SCA_MAC)
    assert p.n_sources == 2
    s0, s1 = p.sources[0], p.sources[1]
    assert s0.shape == capi.SOURCE_BOX and s0.cx == np.float32(0.5) * 24 and s0.hy == np.float32(0.08) * 20
    assert s1.shape == capi.SOURCE_SPHERE and s1.hx == np.float32(0.12) * 24 and s1.temperature == np.float32(0.5)
    ref_occ = wl.add_box(wl.walls_open_top(W, H, D), 8, 10, 9, 11, 5, 8)
    np.testing.assert_array_equal(occ, ref_occ)
    u, v, w = wl.initial_velocity(ref_occ, 3, amp=0.05)
    np.testing.assert_array_equal(st["u"], u)
    np.testing.assert_array_equal(st["v"], v)
    np.testing.assert_array_equal(st["w"], w)
    assert not st["rho"].any() and not st["T"].any()


def test_reference_config_quirks(driver, tmp_path):
    # the reference's own preview config: "step" is not a key (steps stays 20),
    # "inReg_outMAC2" is an unknown advection type, so LoadFromFile fails
    bad = "resolution 16 16 16\nsubSize 2\nsource 0.5 0.1 0.5 0.1 0.05 0.1 0.8 20\nadvVelType inReg_outMAC2\n"
    cfg = tmp_path / "bad.txt"
    cfg.write_text(bad)
    r = subprocess.run([str(driver), "parse", str(cfg), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 3
    ok = "resolution 16 16 16\nsubSize 2\nsource 0.5 0.1 0.5 0.1 0.05 0.1 0.8 20\nstep 30\nvelAttenCoeff 10\n"
    out = run_driver(driver, "parse", ok, tmp_path / "q")
    p, occ, _ = load_setup(out, 16, 16, 16)
    # the reference's default solver is COARSE_OPEN_POISSON_SOR (coarse grid, subSize blocks)
    assert p.substeps == 20 and p.sor_iters == 100 and p.solver == capi.SOLVER_COARSE_OPEN and p.sub_size == 2
    assert p.vel_atten == np.float32(math.exp(np.float32(-0.01) * np.float32(10.0)))
    assert (p.adv_vel_mode, p.adv_sca_mode) == (capi.ADV_VEL_INREG_OUTREG, capi.ADV_SCA_REG)
    assert not occ.any()  # open solver, no internal object
    nosrc = "resolution 16 16 16\nsubSize 2\n"
    cfg.write_text(nosrc)
    assert subprocess.run([str(driver), "parse", str(cfg), str(tmp_path)], capture_output=True).returncode == 3


@pytest.mark.gpu
def test_resident_and_stage_paths_match_oracle(driver, tmp_path, oracle32):
    W, H, D = 24, 20, 16
    run_out = run_driver(driver, "run", CONFIG, tmp_path / "run")
    stage_out = run_driver(driver, "stages", CONFIG, tmp_path / "stages")
    p, occ, st = load_setup(run_out, W, H, D)
    ref = {k: np.ascontiguousarray(v) for k, v in st.items()}
    for i in range(3):
        rc, _ = oracle32.step(W, H, D, ref, occ, p, 1)
        assert rc == 0
        resident = load_di3(run_out / f"frame{i}.di3")
        staged = load_di3(stage_out / f"stage_frame{i}.di3")
        np.testing.assert_array_equal(resident, ref["rho"])
        np.testing.assert_array_equal(staged, ref["rho"])
    fin = load_guide(run_out / "final.guidedat", W, H, D)
    for k in ("u", "v", "w", "T", "rho"):
        np.testing.assert_array_equal(fin[k], ref[k])
    assert float(ref["rho"].sum()) > 0.0


@pytest.mark.gpu
def test_coarse_solver_config_matches_oracle(driver, tmp_path, oracle32):
    """COARSE_CLOSED_POISSON_SOR runs the coarse-grid projection (the open coarse
    solver, as the reference does); blocks with obstacles are least-squares
    solves, so the comparison carries a floating-point tolerance."""
    W, H, D = 24, 20, 16
    cfg = CONFIG.replace("globalGridSolver TOTAL_CLOSED_POISSON_SOR", "globalGridSolver COARSE_CLOSED_POISSON_SOR")
    run_out = run_driver(driver, "run", cfg, tmp_path / "run")
    p, occ, st = load_setup(run_out, W, H, D)
    assert p.solver == capi.SOLVER_COARSE_OPEN and p.sub_size == 4
    ref = {k: np.ascontiguousarray(v) for k, v in st.items()}
    rc, _ = oracle32.step(W, H, D, ref, occ, p, 3)
    assert rc == 0
    fin = load_guide(run_out / "final.guidedat", W, H, D)
    for k in ("u", "v", "w", "T", "rho"):
        assert rel_l2(fin[k], ref[k]) <= 1e-5, k


# moving objects (ZQ_SmokeMovingObject3D.cpp:101-123 file format)
OBJECTS = [
    {"mask": (np.arange(3 * 4 * 5).reshape(3, 4, 5) % 3 != 0), "center": (2, 1, 1), "pos": (6, 5, 5),
     "vels": [(1, 0, 0), (1, 1, 0), (0, 1, -1)]},
    {"mask": np.ones((2, 2, 2), bool), "center": (0, 0, 0), "pos": (15, 12, 9), "vels": [(0, -2, 1)]},
]


def write_objects(path, objs):
    lines = [str(len(objs))]
    for o in objs:
        sz, sy, sx = o["mask"].shape
        lines += [f"{sx} {sy} {sz}", "{} {} {}".format(*o["center"]), "{} {} {}".format(*o["pos"]),
                  str(len(o["vels"]))]
        lines += ["{} {} {}".format(*v) for v in o["vels"]]
        lines.append(" ".join(str(int(b)) for b in o["mask"].ravel()))
    path.write_text("\n".join(lines) + "\n")


def object_track(o, t):
    """(pos, vel) after t calls of UpdateOneStep (ZQ_SmokeMovingObject3D.cpp:83-98)."""
    pos = list(o["pos"])
    for s in range(t):
        if s < len(o["vels"]):
            pos = [a + b for a, b in zip(pos, o["vels"][s])]
    vel = o["vels"][t] if t < len(o["vels"]) else (0, 0, 0)
    return tuple(pos), tuple(vel)


def test_load_moving_objects(driver, tmp_path):
    f = tmp_path / "objs.txt"
    write_objects(f, OBJECTS)
    r = subprocess.run([str(driver), "objects", str(f), str(tmp_path)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    rows = (tmp_path / "objects.txt").read_text().split("\n")
    assert int(rows[0]) == 2
    for o, row in zip(OBJECTS, rows[1:]):
        vals = [int(x) for x in row.split()]
        sz, sy, sx = o["mask"].shape
        assert vals[:8] == [sx, sy, sz, *o["center"], len(o["vels"]), int(o["mask"].sum())]
        for t in range(4):
            pos, vel = object_track(o, t)
            assert tuple(vals[8 + 6 * t: 11 + 6 * t]) == pos and tuple(vals[11 + 6 * t: 14 + 6 * t]) == vel
    # a truncated file fails
    f.write_text("1\n2 2 2\n0 0 0\n1 1 1\n1\n0 0 0\n1 1 1\n")
    assert subprocess.run([str(driver), "objects", str(f), str(tmp_path)], capture_output=True).returncode == 3


@pytest.mark.gpu
def test_moving_objects_match_oracle(driver, tmp_path, oracle32):
    """useMovingObject: the objects are stamped at Init, again before every
    frame from the second on, and advanced after each frame; the resident class
    path and the free-function path (ZQ_ApplyMovingObject3D) both equal the
    oracle's stamp + step sequence bit for bit."""
    W, H, D = 24, 20, 16
    objf = tmp_path / "objs.txt"
    write_objects(objf, OBJECTS)
    cfg = CONFIG.replace("stepTime 0.05", "stepTime 0.02") + f"useMovingObject true\nmovingObjectFile {objf}\n"
    pre = run_driver(driver, "parse", cfg, tmp_path / "pre")
    run_out = run_driver(driver, "run", cfg, tmp_path / "run")
    stage_out = run_driver(driver, "stages", cfg, tmp_path / "stages")
    p, occ0, st0 = load_setup(pre, W, H, D)
    ref = {k: np.ascontiguousarray(v).copy() for k, v in st0.items()}
    occ = np.ascontiguousarray(occ0).copy()

    def stamp(t):
        objs = []
        for o in OBJECTS:
            pos, vel = object_track(o, t)
            objs.append({"mask": o["mask"], "center": o["center"], "pos": pos, "vel": vel})
        oracle32.stamp_objects(W, H, D, ref, occ, objs, 2, p)   # wallsExceptTop: all walls but y = H-1

    stamp(0)
    _, occ_init, st_init = load_setup(run_out, W, H, D)
    np.testing.assert_array_equal(occ_init, occ)
    for k in ("u", "v", "w"):
        np.testing.assert_array_equal(st_init[k], ref[k])
    assert int(2 * np.float64(np.float32(1.0 / 24) / np.float32(0.02))) != 0   # the stamped velocities are not zero
    for i in range(3):
        if i > 0:
            stamp(i)
        rc, _ = oracle32.step(W, H, D, ref, occ, p, 1)
        assert rc == 0
        np.testing.assert_array_equal(load_di3(run_out / f"frame{i}.di3"), ref["rho"])
        np.testing.assert_array_equal(load_di3(stage_out / f"stage_frame{i}.di3"), ref["rho"])
    fin = load_guide(run_out / "final.guidedat", W, H, D)
    for k in ("u", "v", "w", "T", "rho"):
        np.testing.assert_array_equal(fin[k], ref[k])


# headless viewer (ZQ_LoadVolume3D / ZQ_RenderSequence3D)
def write_di3(path, vol, channels=1):
    D, H, W = vol.shape[:3]
    with open(path, "wb") as f:
        f.write(b"float" + b"\0" * 11)
        f.write(np.array([W, H, D, channels], np.int32).tobytes())
        f.write(b"\0")
        f.write(np.ascontiguousarray(vol, np.float32).tobytes())


def read_vol(outdir):
    W, H, D = np.fromfile(outdir / "vol.bin", np.int32)
    return np.fromfile(outdir / "vol_data.bin", np.float32).reshape(D, H, W)


def test_load_volume_formats(driver, tmp_path):
    rng = np.random.default_rng(2)
    vol = rng.random((5, 4, 6), dtype=np.float32)
    write_di3(tmp_path / "a.di3", vol)
    r = subprocess.run([str(driver), "loadvol", str(tmp_path / "a.di3"), str(tmp_path)], capture_output=True)
    assert r.returncode == 0
    np.testing.assert_array_equal(read_vol(tmp_path), vol)
    # two channels are averaged into one
    two = np.stack([vol, 3 * vol], axis=-1)
    write_di3(tmp_path / "b.di3", two, channels=2)
    assert subprocess.run([str(driver), "loadvol", str(tmp_path / "b.di3"), str(tmp_path)]).returncode == 0
    np.testing.assert_array_equal(read_vol(tmp_path), ((vol + 3 * vol) / np.float32(2)).astype(np.float32))
    # raw N^3 floats: the viewer swaps the first and last axes
    N = 5
    raw = rng.random((N, N, N), dtype=np.float32)
    raw.tofile(tmp_path / "c.dat")
    assert subprocess.run([str(driver), "loadvol", str(tmp_path / "c.dat"), str(tmp_path), str(N)]).returncode == 0
    np.testing.assert_array_equal(read_vol(tmp_path), raw.transpose(2, 1, 0))
    # ZQlib formats and truncated files are refused
    (tmp_path / "d.zqci").write_bytes(b"x")
    assert subprocess.run([str(driver), "loadvol", str(tmp_path / "d.zqci"), str(tmp_path)]).returncode == 3
    (tmp_path / "e.di3").write_bytes((tmp_path / "a.di3").read_bytes()[:-8])
    assert subprocess.run([str(driver), "loadvol", str(tmp_path / "e.di3"), str(tmp_path)]).returncode == 3


def ppm_of(rgba):
    rgb = (np.clip(rgba[..., :3], 0.0, 1.0)[::-1] * np.float32(255.0) + np.float32(0.5)).astype(np.uint8)
    return b"P6\n%d %d\n255\n" % (rgb.shape[1], rgb.shape[0]) + rgb.tobytes()


@pytest.mark.gpu
def test_render_sequence_matches_oracle(driver, tmp_path, oracle32):
    """The viewer's sequence mode without a window: two .di3 frames and one raw
    frame in the start-up view, PPM bytes equal to the oracle's render."""
    rng = np.random.default_rng(4)
    frames = [rng.random((12, 16, 20), dtype=np.float32) * 0.2, rng.random((12, 16, 20), dtype=np.float32)]
    for n, v in enumerate(frames):
        write_di3(tmp_path / f"frame{n + 3}.di3", v)
    out = tmp_path / "out"
    out.mkdir()
    r = subprocess.run([str(driver), "sequence", str(tmp_path), str(out), "frame", "3", "2", ".di3", "0", "40", "30"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    for n, v in enumerate(frames):
        cam = capi.default_camera(40, 30, 20, 16, 12)
        ref = oracle32.render(v, cam)
        assert (out / f"render{n + 3}.ppm").read_bytes() == ppm_of(ref)
    N = 8
    raw = rng.random((N, N, N), dtype=np.float32)
    raw.tofile(tmp_path / "raw0.dat")
    r = subprocess.run([str(driver), "sequence", str(tmp_path), str(out), "raw", "0", "1", ".dat", str(N), "24", "24"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    ref = oracle32.render(np.ascontiguousarray(raw.transpose(2, 1, 0)), capi.default_camera(24, 24, N, N, N))
    assert (out / "render0.ppm").read_bytes() == ppm_of(ref)


@pytest.mark.parametrize("name,walls_except_top,expect", [
    ("TOTAL_OPEN_POISSON_SOR", "false", capi.SOLVER_OPEN),
    ("TOTAL_CLOSED_POISSON_SOR", "false", capi.SOLVER_CLOSED),
    ("TOTAL_CLOSED_POISSON_SOR", "true", capi.SOLVER_OPEN),
    ("CLOSED_OCTREE_POISSON_SOR", "false", capi.SOLVER_CLOSED),
    ("OPEN_OCTREE_POISSON", "false", capi.SOLVER_OPEN),
    ("COARSE_OPEN_POISSON_SOR", "false", capi.SOLVER_COARSE_OPEN),
    ("COARSE_CLOSED_POISSON_SOR", "false", capi.SOLVER_COARSE_OPEN),
    ("COARSE_CLOSED_FLUX_SOR", "false", capi.SOLVER_CLOSED),
    ("NOT_A_SOLVER", "false", capi.SOLVER_OPEN),
])
def test_global_solver_names_map_to_runtime_solver(driver, tmp_path, name, walls_except_top, expect):
    """globalGridSolver names (ZQ_SmokeSimulationPara3D's parser): both coarse
    Poisson settings run the open coarse solver, as ZQ_TotalProjection3D does
    (Utils3D:3731-3745); every other setting the fine-grid SOR of its open or
    closed kind (open with wallsExceptTop); an unknown name falls back to
    OPEN_FLUX, an open solver."""
    cfg = CONFIG.replace("wallsExceptTop true", "wallsExceptTop " + walls_except_top) \
                .replace("globalGridSolver TOTAL_CLOSED_POISSON_SOR", "globalGridSolver " + name)
    out = run_driver(driver, "parse", cfg, tmp_path / "s")
    p, occ, _ = load_setup(out, 24, 20, 16)
    assert p.solver == expect
    if expect == capi.SOLVER_CLOSED:
        np.testing.assert_array_equal(occ, wl.add_box(wl.walls_closed(24, 20, 16), 8, 10, 9, 11, 5, 8))
