"""Moving voxel objects (ZQ_ApplyMovingObject3D, Utils3D:1933-2046): the
oracle's restatement pinned by known answers (CPU) and the GPU stamping
(zqs_grid_stamp_objects) bit for bit against it, followed by steps."""
import numpy as np
import pytest

from zq_smokesimulation_gb300 import capi
from zq_smokesimulation_gb300 import workloads as wl

W, H, D = 20, 16, 12


def objects(seed=4):
    rng = np.random.default_rng(seed)
    a = rng.random((3, 4, 5)) < 0.6            # (sz, sy, sx)
    b = np.ones((2, 3, 3), bool)
    b[1, 1, 1] = False
    return [{"mask": a, "center": (2, 1, 1), "pos": (8, 6, 5), "vel": (1, -2, 0)},
            {"mask": b, "center": (1, 1, 0), "pos": (19, 7, 11), "vel": (0, 1, 3)},   # partly outside
            {"mask": a[:, :2, :3], "center": (0, 0, 0), "pos": (9, 6, 5), "vel": (-1, 0, 2)}]  # overlaps the first


def base(closed=False):
    w = wl.small_case(W, H, D, K=12, vel_amp=0.3)
    w.params.solver = capi.SOLVER_CLOSED if closed else capi.SOLVER_OPEN
    return w


def test_single_voxel_known_answer(oracle32):
    w = base()
    p = w.params
    st = oracle32.state(w)
    occ = np.ascontiguousarray(w.occ, np.uint8).copy()
    obj = [{"mask": np.ones((1, 1, 1), bool), "center": (0, 0, 0), "pos": (5, 4, 3), "vel": (2, -1, 1)}]
    oracle32.stamp_objects(W, H, D, st, occ, obj, False, p)
    assert occ.sum() == 1 and occ[3, 4, 5] == 1          # every other cell cleared (static obstacles too)
    scale = float(np.float64(np.float32(p.voxel_size) / np.float32(p.step_time)))
    cu, cv, cw = int(2 * scale), int(-1 * scale), int(1 * scale)
    assert st["u"][3, 4, 5] == cu and st["u"][3, 4, 6] == cu
    assert st["v"][3, 4, 5] == cv and st["v"][3, 5, 5] == cv
    assert st["w"][3, 4, 5] == cw and st["w"][4, 4, 5] == cw


def test_closed_walls_known_answer(oracle32):
    w = base(closed=True)
    st = oracle32.state(w)
    occ = np.zeros((D, H, W), np.uint8)
    oracle32.stamp_objects(W, H, D, st, occ, [], True, w.params)
    ref = np.zeros((D, H, W), np.uint8)
    ref[0], ref[-1], ref[:, 0], ref[:, -1], ref[:, :, 0], ref[:, :, -1] = 1, 1, 1, 1, 1, 1
    np.testing.assert_array_equal(occ, ref)
    # 2: the open-top walls (every wall but the y = H-1 layer)
    oracle32.stamp_objects(W, H, D, st, occ, [], 2, w.params)
    np.testing.assert_array_equal(occ, wl.walls_open_top(W, H, D))


@pytest.mark.gpu
def test_stamp_argument_checks(zqs_lib):
    g = capi.Grid(W, H, D)
    with pytest.raises(capi.ZQSError) as e:      # no parameters yet: h / dt unknown
        g.stamp_objects([])
    assert e.value.code == capi.ZQS_ENOTREADY
    g.set_params(base().params)
    with pytest.raises(capi.ZQSError) as e:
        g.stamp_objects([], closed_walls=3)
    assert e.value.code == capi.ZQS_EINVAL
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("closed", [0, 1, 2])
def test_stamp_matches_oracle_then_steps(zqs_lib, oracle32, closed):
    w = base(closed == 1)
    g = capi.Grid(W, H, D)
    g.set_params(w.params)
    g.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
    objs = objects()
    g.stamp_objects(objs, closed_walls=closed)
    st = oracle32.state(w)
    occ = np.ascontiguousarray(w.occ, np.uint8).copy()
    oracle32.stamp_objects(W, H, D, st, occ, objs, closed, w.params)
    np.testing.assert_array_equal(g.download(capi.FIELD_OCCUPANCY), occ)
    out = g.state()
    for k in ("u", "v", "w"):
        np.testing.assert_array_equal(out[k], st[k])
    g.step(2)
    rc, _ = oracle32.step(W, H, D, st, occ, w.params, 2)
    assert rc == 0
    out = g.state()
    for k in ("u", "v", "w", "T", "rho"):
        np.testing.assert_array_equal(out[k], st[k])
    g.close()


@pytest.mark.gpu
@pytest.mark.parametrize("solver", [capi.SOLVER_OPEN, capi.SOLVER_CLOSED])
def test_moving_sequence_matches_oracle(zqs_lib, oracle32, solver):
    """Objects re-stamped between steps at moved positions: cells that turn
    solid carry the previous step's pressure, which the flag rebuild clears
    (the SOR sums all six neighbours), so every step stays bit-identical."""
    w = base(solver == capi.SOLVER_CLOSED)
    closed = 1 if solver == capi.SOLVER_CLOSED else 0
    g = capi.Grid(W, H, D)
    g.set_params(w.params)
    g.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
    st = oracle32.state(w)
    occ = np.ascontiguousarray(w.occ, np.uint8).copy()
    objs = objects()
    for t in range(4):
        moved = [dict(o, pos=tuple(a + t * b for a, b in zip(o["pos"], o["vel"]))) for o in objs]
        g.stamp_objects(moved, closed_walls=closed)
        oracle32.stamp_objects(W, H, D, st, occ, moved, closed, w.params)
        g.step(1)
        rc, _ = oracle32.step(W, H, D, st, occ, w.params, 1)
        assert rc == 0
        out = g.state()
        for k in ("u", "v", "w", "T", "rho"):
            np.testing.assert_array_equal(out[k], st[k], err_msg=f"step {t} field {k}")
    g.close()


def python_stamp(W, H, D, u, v, w, objs, closed, h, dt):
    """ZQ_ApplyMovingObject3D (Utils3D:1933-2046) restated in plain Python: the
    occupancy is cleared, each object's solid in-domain voxels occupy their
    cell and set its six faces to int(vel * (double)(h / dt)), then the closed
    solvers' walls (mode 2: all but the y = H-1 layer) are occupied."""
    occ = np.zeros((D, H, W), np.uint8)
    scale = float(np.float32(h) / np.float32(dt))
    for o in objs:
        m = np.asarray(o["mask"], bool)
        sz, sy, sx = m.shape
        cx, cy, cz = o["center"]
        px, py, pz = o["pos"]
        vel = [int(c * scale) for c in o["vel"]]
        for k in range(sz):
            for j in range(sy):
                for i in range(sx):
                    if not m[k, j, i]:
                        continue
                    x, y, z = i + px - cx, j + py - cy, k + pz - cz
                    if 0 <= x < W and 0 <= y < H and 0 <= z < D:
                        occ[z, y, x] = 1
                        u[z, y, x] = u[z, y, x + 1] = vel[0]
                        v[z, y, x] = v[z, y + 1, x] = vel[1]
                        w[z, y, x] = w[z + 1, y, x] = vel[2]
    if closed:
        occ[:, :, 0] = occ[:, :, W - 1] = 1
        occ[:, 0, :] = 1
        if closed == 1:
            occ[:, H - 1, :] = 1
        occ[0, :, :] = occ[D - 1, :, :] = 1
    return occ


@pytest.mark.parametrize("closed", [0, 1, 2])
def test_oracle_stamp_matches_python_restatement(oracle32, closed):
    w = base(closed == 1)
    p = w.params
    st = oracle32.state(w)
    occ = np.ascontiguousarray(w.occ, np.uint8).copy()
    objs = objects(seed=11)
    oracle32.stamp_objects(W, H, D, st, occ, objs, closed, p)
    ref = oracle32.state(w)
    ref_occ = python_stamp(W, H, D, ref["u"], ref["v"], ref["w"], objs, closed, p.voxel_size, p.step_time)
    np.testing.assert_array_equal(occ, ref_occ)
    for k in ("u", "v", "w"):
        np.testing.assert_array_equal(st[k], ref[k])
