"""Known-answer tests of the CPU oracle (no GPU).

The reference ships no tests or golden outputs, so the oracle is pinned by
(1) analytic known answers, (2) small pure-Python restatements of the
reference loops that the C++ oracle must match bit for bit, (3) FP32 vs FP64
agreement, and (4) the committed golden fixtures under tests/golden/.
"""
import math

import numpy as np
import pytest

from conftest import rel_l2
from zq_smokesimulation_gb300 import capi
from zq_smokesimulation_gb300 import workloads as wl


def free_occ(W, H, D):
    return np.zeros((D, H, W), np.uint8)


def test_mac_to_regular_constant_and_linear(oracle64):
    W, H, D = 6, 5, 4
    i = np.arange(W + 1, dtype=np.float64)
    u = np.broadcast_to(0.5 + 2.0 * i, (D, H, W + 1)).copy()
    v = np.full((D, H + 1, W), 3.0)
    w = np.full((D + 1, H, W), -1.25)
    c4 = oracle64.mac_to_regular4(W, H, D, u, v, w)
    assert np.all(c4[..., 1] == 3.0) and np.all(c4[..., 2] == -1.25) and np.all(c4[..., 3] == 0.0)
    np.testing.assert_allclose(c4[..., 0], np.broadcast_to(0.5 + 2.0 * (np.arange(W) + 0.5), (D, H, W)))
    u2, v2, w2 = oracle64.regular4_to_mac(W, H, D, c4)
    # interior faces of a linear field come back exactly; domain faces copy the inner centre
    np.testing.assert_allclose(u2[:, :, 1:W], u[:, :, 1:W], rtol=0, atol=1e-14)
    np.testing.assert_allclose(u2[:, :, 0], c4[:, :, 0, 0])
    np.testing.assert_allclose(u2[:, :, W], c4[:, :, W - 1, 0])
    assert np.all(v2 == 3.0) and np.all(w2 == -1.25)


@pytest.mark.parametrize("mode", [capi.ADV_VEL_INMAC_OUTMAC, capi.ADV_VEL_INREG_OUTMAC, capi.ADV_VEL_INREG_OUTREG])
def test_advect_velocity_constant_field_invariant(oracle32, mode):
    W, H, D = 7, 6, 5
    p = wl.smoke_params(W, 1, substeps=5)
    st = {"u": np.full((D, H, W + 1), 0.3, np.float32), "v": np.full((D, H + 1, W), -0.2, np.float32),
          "w": np.full((D + 1, H, W), 0.1, np.float32)}
    before = {k: v.copy() for k, v in st.items()}
    assert oracle32.advect_velocity(W, H, D, st, free_occ(W, H, D), p, mode) == 0
    for k in st:
        assert np.array_equal(st[k], before[k]), k


def test_advect_zero_velocity_is_identity(oracle32):
    w = wl.small_case(8, 7, 6, vel_amp=0.0)
    st = oracle32.state(w)
    T0, R0 = st["T"].copy(), st["rho"].copy()
    assert oracle32.advect_scalar(w.W, w.H, w.D, st, w.occ, w.params, capi.ADV_SCA_MAC) == 0
    assert np.array_equal(st["T"], T0) and np.array_equal(st["rho"], R0)
    st2 = oracle32.state(w)
    u0 = st2["u"].copy()
    assert oracle32.advect_velocity(w.W, w.H, w.D, st2, w.occ, w.params, capi.ADV_VEL_INMAC_OUTMAC) == 0
    assert np.array_equal(st2["u"], u0)


def _translation_case(substeps, full):
    W, H, D = 16, 6, 6
    p = wl.smoke_params(W, 1, substeps=substeps)
    p.voxel_size = 1.0 / W
    p.step_time = 2.0 * p.voxel_size   # with u = 1: (u*dt)/h = 2 cells in total
    p.backtrace_full = 1 if full else 0
    st = {"u": np.ones((D, H, W + 1), np.float32), "v": np.zeros((D, H + 1, W), np.float32),
          "w": np.zeros((D + 1, H, W), np.float32)}
    T = np.random.default_rng(3).random((D, H, W)).astype(np.float32)
    st["T"], st["rho"] = T.copy(), T.copy()
    return W, H, D, p, st, T


def test_backtrace_reference_rule_uses_point_before_last_move(oracle32):
    # substeps=2: the reference samples after 1 of the 2 moves -> a 1-cell shift
    W, H, D, p, st, T = _translation_case(2, False)
    oracle32.advect_scalar(W, H, D, st, free_occ(W, H, D), p, capi.ADV_SCA_MAC)
    np.testing.assert_array_equal(st["T"][:, :, 4:W - 1], T[:, :, 3:W - 2])
    # substeps=1: no move survives -> identity (the documented reference quirk)
    W, H, D, p, st, T = _translation_case(1, False)
    oracle32.advect_scalar(W, H, D, st, free_occ(W, H, D), p, capi.ADV_SCA_MAC)
    np.testing.assert_array_equal(st["T"], T)


def test_backtrace_full_rule_uses_final_point(oracle32):
    W, H, D, p, st, T = _translation_case(1, True)
    oracle32.advect_scalar(W, H, D, st, free_occ(W, H, D), p, capi.ADV_SCA_MAC)
    np.testing.assert_array_equal(st["T"][:, :, 4:W - 1], T[:, :, 2:W - 3])


def test_linear_field_interpolates_exactly(oracle64):
    W, H, D = 12, 10, 8
    p = wl.smoke_params(W, 1, substeps=3)
    p.step_time = 0.37 * p.voxel_size
    occ = free_occ(W, H, D)
    k, j, i = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    T = 0.25 + 0.5 * (i + 0.5) - 0.125 * (j + 0.5) + 0.0625 * (k + 0.5)
    st = {"u": np.full((D, H, W + 1), 0.7), "v": np.full((D, H + 1, W), 0.4), "w": np.full((D + 1, H, W), -0.3),
          "T": T.copy(), "rho": T.copy()}
    oracle64.advect_scalar(W, H, D, st, occ, p, capi.ADV_SCA_MAC)
    dt_sub = float(p.step_time) / 3.0                      # the params hold float32 values
    shift = 2 * dt_sub / float(p.voxel_size) * np.array([0.7, 0.4, -0.3])   # 2 of 3 moves survive
    exp = T - (0.5 * shift[0] - 0.125 * shift[1] + 0.0625 * shift[2])
    sl = (slice(2, D - 2), slice(2, H - 2), slice(2, W - 2))
    np.testing.assert_allclose(st["T"][sl], exp[sl], rtol=0, atol=1e-12)


def test_vorticity_of_rigid_rotation(oracle64):
    W = H = D = 9
    h = 1.0 / W
    Om = 0.75
    # u_c = -Om*(y - yc), v_c = Om*(x - xc) (physical units), on faces
    y_u = (np.arange(H) + 0.5) * h - 0.5
    x_v = (np.arange(W) + 0.5) * h - 0.5
    u = np.broadcast_to((-Om * y_u)[None, :, None], (D, H, W + 1)).copy()
    v = np.broadcast_to((Om * x_v)[None, None, :], (D, H + 1, W)).copy()
    w = np.zeros((D + 1, H, W))
    vort, vs = oracle64.vorticity(W, H, D, u, v, w, h)
    inner = (slice(1, D - 1), slice(1, H - 1), slice(1, W - 1))
    np.testing.assert_allclose(vort[inner][..., 2], 2 * Om, rtol=1e-12)
    np.testing.assert_allclose(vort[inner][..., 0], 0, atol=1e-12)
    np.testing.assert_allclose(vs[inner], 2 * Om, rtol=1e-12)
    assert np.all(vort[0] == 0) and np.all(vs[:, :, 0] == 0)   # boundary cells stay zero


def _gradient_field(pstar, occ):
    """Live-face gradient of pstar with p = 0 outside (open rule)."""
    D, H, W = occ.shape
    lu, lv, lw = wl.live_faces(occ)
    pp = np.pad(pstar, 1)
    u = (pp[1:-1, 1:-1, 1:] - pp[1:-1, 1:-1, :-1]) * lu
    v = (pp[1:-1, 1:, 1:-1] - pp[1:-1, :-1, 1:-1]) * lv
    w = (pp[1:, 1:-1, 1:-1] - pp[:-1, 1:-1, 1:-1]) * lw
    return u, v, w


def test_sor_recovers_manufactured_pressure(oracle64):
    W, H, D = 10, 9, 8
    occ = wl.walls_open_top(W, H, D)
    wl.add_box(occ, 4, 5, 4, 5, 3, 4)
    rng = np.random.default_rng(11)
    pstar = rng.standard_normal((D, H, W)) * (occ == 0)
    u, v, w = _gradient_field(pstar, occ)
    p = wl.smoke_params(W, 3000, omega=1.8)
    st = {"u": u.copy(), "v": v.copy(), "w": w.copy()}
    pr, div, stats = oracle64.project(W, H, D, st, occ, p, want=True)
    np.testing.assert_allclose(pr, pstar, atol=1e-9)
    for k in ("u", "v", "w"):
        assert np.abs(st[k]).max() < 1e-9
    assert stats.max_abs_div < 1e-9 and stats.residual_l2 < 1e-9


def test_closed_solver_removes_mean_divergence(oracle64):
    w_ = wl.small_case(9, 8, 7, closed=True, K=4000, vel_amp=0.2)
    st = oracle64.state(w_)
    w_.params.omega = 1.7
    pr, div, stats = oracle64.project(w_.W, w_.H, w_.D, st, w_.occ, w_.params, want=True)
    u, v, w = st["u"], st["v"], st["w"]
    d = (u[:, :, 1:] - u[:, :, :-1]) + (v[:, 1:, :] - v[:, :-1, :]) + (w[1:] - w[:-1])
    free = w_.occ == 0
    np.testing.assert_allclose(d[free], stats.div_mean_removed, atol=1e-9)
    assert stats.residual_l2 < 1e-9


def _fma(a, b, c):
    """Correctly rounded a*b + c in double (exact rational arithmetic)."""
    from fractions import Fraction
    return float(Fraction(a) * Fraction(b) + Fraction(c))


def _py_sor(div, occ, K, omega, open_):
    """Pure-Python red-black SOR on a tiny grid (same operation order: the
    neighbour sum ((x- + x+) + (y- + y+)) + (z- + z+) with 0 for excluded
    neighbours, then fma(omega/cnt, s - div, (1-omega) p))."""
    D, H, W = occ.shape
    p = np.zeros((D, H, W))
    nb = [(-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)]
    for _ in range(K):
        for colour in (0, 1):
            for k in range(D):
                for j in range(H):
                    for i in range(W):
                        if (i + j + k) % 2 != colour or occ[k, j, i]:
                            continue
                        vals, cnt = [], 0
                        for di, dj, dk in nb:
                            a, b, c = i + di, j + dj, k + dk
                            val = 0.0
                            if 0 <= a < W and 0 <= b < H and 0 <= c < D:
                                if not occ[c, b, a]:
                                    val = p[c, b, a]
                                    cnt += 1
                            elif open_:
                                cnt += 1
                            vals.append(val)
                        if cnt == 0:
                            continue
                        s = ((vals[0] + vals[1]) + (vals[2] + vals[3])) + (vals[4] + vals[5])
                        p[k, j, i] = _fma(omega / cnt, s - div[k, j, i], (1.0 - omega) * p[k, j, i])
    return p


@pytest.mark.parametrize("open_,omega", [(True, 1.0), (True, 1.9), (False, 1.3)])
def test_sor_matches_pure_python_restatement(oracle64, open_, omega):
    W, H, D = 5, 4, 4
    occ = np.zeros((D, H, W), np.uint8)
    occ[1, 1, 2] = 1
    occ[2, 3, 0] = 1
    rng = np.random.default_rng(5)
    st = {"u": rng.standard_normal((D, H, W + 1)), "v": rng.standard_normal((D, H + 1, W)),
          "w": rng.standard_normal((D + 1, H, W))}
    lu, lv, lw = wl.live_faces(occ)
    for k_, m in zip(("u", "v", "w"), (lu, lv, lw)):
        st[k_] = st[k_] * m
    p = wl.smoke_params(W, 3, omega=omega, solver=capi.SOLVER_OPEN if open_ else capi.SOLVER_CLOSED)
    pr, div, _ = oracle64.project(W, H, D, {k: v.copy() for k, v in st.items()}, occ, p, want=True)
    u, v, w = st["u"], st["v"], st["w"]
    d = ((((u[:, :, 1:] - u[:, :, :-1]) + v[:, 1:, :]) - v[:, :-1, :]) + w[1:]) - w[:-1]
    d = d * (occ == 0)
    if not open_:
        # FP64 mean: per-plane sequential partial sums combined in plane order
        total, n = 0.0, 0
        for k in range(D):
            part = 0.0
            for j in range(H):
                for i in range(W):
                    if not occ[k, j, i]:
                        part += d[k, j, i]
                        n += 1
            total += part
        d = d - (total / n) * (occ == 0)
    np.testing.assert_array_equal(div, d)
    np.testing.assert_array_equal(pr, _py_sor(d, occ, 3, float(p.omega), open_))  # omega as stored (float32)


def _py_backtrace_mac(u, v, w, occ, start, steps, dt, h):
    D, H, W = occ.shape

    def tri(f, g):
        nz, ny, nx = f.shape
        idx, ts = [], []
        for gg, n in zip(g, (nx, ny, nz)):
            gg = min(max(gg, -1.0), float(n))
            fl = math.floor(gg)
            ts.append(gg - fl)
            idx.append((min(max(fl, 0), n - 1), min(max(fl + 1, 0), n - 1)))
        (x0, x1), (y0, y1), (z0, z1) = idx
        tx, ty, tz = ts
        L = lambda a, b, t: a + t * (b - a)
        c00 = L(f[z0, y0, x0], f[z0, y0, x1], tx)
        c10 = L(f[z0, y1, x0], f[z0, y1, x1], tx)
        c01 = L(f[z1, y0, x0], f[z1, y0, x1], tx)
        c11 = L(f[z1, y1, x0], f[z1, y1, x1], tx)
        return L(L(c00, c10, ty), L(c01, c11, ty), tz)

    def vel(x, y, z):
        return (tri(u, (x, y - 0.5, z - 0.5)), tri(v, (x - 0.5, y, z - 0.5)), tri(w, (x - 0.5, y - 0.5, z)))

    x, y, z = start
    vx, vy, vz = vel(x, y, z)
    last = (x, y, z)
    for _ in range(steps):
        if not (0 <= x <= W and 0 <= y <= H and 0 <= z <= D):
            break
        if occ[min(max(int(math.floor(z)), 0), D - 1), min(max(int(math.floor(y)), 0), H - 1),
               min(max(int(math.floor(x)), 0), W - 1)]:
            break
        last = (x, y, z)
        x, y, z = x - (vx * dt) / h, y - (vy * dt) / h, z - (vz * dt) / h
        vx, vy, vz = vel(x, y, z)
    return last, tri


def test_scalar_advection_matches_pure_python_restatement(oracle64):
    w_ = wl.small_case(7, 6, 5, vel_amp=0.4, substeps=3)
    st = {k: np.asarray(v, np.float64).copy() for k, v in w_.state().items()}
    T0 = st["T"].copy()
    oracle64.advect_scalar(w_.W, w_.H, w_.D, st, w_.occ, w_.params, capi.ADV_SCA_MAC)
    dt = float(w_.params.step_time) / w_.params.substeps
    h = float(np.float32(w_.params.voxel_size))
    for (k, j, i) in [(0, 0, 0), (2, 3, 4), (4, 5, 6), (1, 2, 3), (3, 1, 5)]:
        last, tri = _py_backtrace_mac(st["u"], st["v"], st["w"], w_.occ, (i + 0.5, j + 0.5, k + 0.5),
                                      w_.params.substeps, dt, h)
        exp = tri(T0, (last[0] - 0.5, last[1] - 0.5, last[2] - 0.5))
        assert st["T"][k, j, i] == exp


def test_fp32_and_fp64_oracles_agree_over_steps(oracle32, oracle64):
    w_ = wl.small_case(12, 12, 10, K=30, substeps=4)
    s32, s64 = oracle32.state(w_), oracle64.state(w_)
    oracle32.step(w_.W, w_.H, w_.D, s32, w_.occ, w_.params, 5)
    oracle64.step(w_.W, w_.H, w_.D, s64, w_.occ, w_.params, 5)
    for k in ("u", "v", "w", "rho", "T"):
        assert rel_l2(s32[k], s64[k]) < 1e-5, k


def test_reinject_box_and_sphere(oracle32):
    W, H, D = 10, 9, 8
    p = wl.smoke_params(W, 1)
    p.set_sources([wl.sphere(5.0, 3.0, 4.0, 2.2, 0.8, 0.6), wl.box(2.0, 6.0, 3.0, 1.0, 0.5, 1.5, 0.3, 0.2)])
    st = {"T": np.zeros((D, H, W), np.float32), "rho": np.zeros((D, H, W), np.float32)}
    oracle32.reinject(W, H, D, st, p)
    k, j, i = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    x, y, z = (i + np.float32(0.5)).astype(np.float32), (j + np.float32(0.5)).astype(np.float32), \
        (k + np.float32(0.5)).astype(np.float32)
    dx, dy, dz = x - np.float32(5), y - np.float32(3), z - np.float32(4)
    sph = (dx * dx + dy * dy) + dz * dz <= np.float32(2.2) * np.float32(2.2)
    bx = (np.abs(x - 2) <= 1.0) & (np.abs(y - 6) <= 0.5) & (np.abs(z - 3) <= 1.5)
    exp_rho = np.where(bx, np.float32(0.3), np.where(sph, np.float32(0.8), 0)).astype(np.float32)
    assert np.array_equal(st["rho"], exp_rho)
    assert sph.sum() > 10 and bx.sum() > 0


def test_force_only_buoyancy_without_confinement(oracle64):
    W, H, D = 6, 7, 5
    occ = wl.walls_open_top(W, H, D)
    p = wl.smoke_params(W, 1)
    p.confine = 0.0
    rng = np.random.default_rng(2)
    st = {"u": np.zeros((D, H, W + 1)), "v": np.zeros((D, H + 1, W)), "w": np.zeros((D + 1, H, W)),
          "T": rng.random((D, H, W)), "rho": rng.random((D, H, W))}
    oracle64.add_force(W, H, D, st, occ, p)
    f = float(p.buoyancy) * (st["T"] - float(p.tamb)) - float(np.float32(p.gravity)) * st["rho"]
    lu, lv, lw = wl.live_faces(occ)
    dt = float(np.float32(p.step_time))
    exp = np.zeros((D, H + 1, W))
    exp[:, 1:H, :] = dt * 0.5 * (f[:, 1:, :] + f[:, :-1, :])
    exp[:, H, :] = dt * f[:, H - 1, :]
    exp[:, 0, :] = dt * f[:, 0, :]
    np.testing.assert_allclose(st["v"], exp * lv, rtol=1e-12, atol=1e-15)
    assert np.all(st["u"] == 0) and np.all(st["w"] == 0)


def test_golden_fixtures(oracle32, oracle64):
    import json
    from pathlib import Path
    gdir = Path(__file__).parent / "golden"
    files = sorted(gdir.glob("*.npz"))
    assert files, "no golden fixtures committed"
    for f in files:
        g = np.load(f)
        meta = json.loads(str(g["meta"]))
        w_ = wl.small_case(*meta["dims"], seed=meta["seed"], K=meta["K"], substeps=meta["substeps"],
                           closed=meta["closed"], vel_mode=meta["vel_mode"], sca_mode=meta["sca_mode"])
        for o, tag in ((oracle32, "f32"), (oracle64, "f64")):
            st = o.state(w_)
            o.step(w_.W, w_.H, w_.D, st, w_.occ, w_.params, meta["steps"])
            for k in ("u", "v", "w", "T", "rho"):
                ref = g[f"{tag}_{k}"]
                if tag == "f32":
                    assert np.array_equal(st[k], ref), (f.name, k)
                else:
                    np.testing.assert_allclose(st[k], ref, rtol=0, atol=1e-13, err_msg=f"{f.name} {k}")


def _py_advect_scalar_mac(phi, u, v, w, occ, steps, dt, h):
    """One semi-Lagrangian pass of a cell field with MAC velocity (every cell
    backtraced from its centre, sampled at the last accepted point)."""
    D, H, W = occ.shape
    out = np.empty_like(phi)
    for k in range(D):
        for j in range(H):
            for i in range(W):
                last, tri = _py_backtrace_mac(u, v, w, occ, (i + 0.5, j + 0.5, k + 0.5), steps, dt, h)
                out[k, j, i] = tri(phi, (last[0] - 0.5, last[1] - 0.5, last[2] - 0.5))
    return out


def test_scalar_bfecc_matches_pure_python_restatement(oracle64):
    """cu_Advect_Scalar_MAC_Velocity_BFECC (Adv3D:1586-1648): forward pass,
    a pass back with the negated velocity, input = input*1.5 - back*0.5
    (Input_Increment_Kernel, Adv3D:56-64, in double), forward pass again."""
    w_ = wl.small_case(6, 5, 4, vel_amp=0.4, substeps=2)
    st = {k: np.asarray(v, np.float64).copy() for k, v in w_.state().items()}
    T0 = st["T"].copy()
    assert oracle64.advect_scalar(w_.W, w_.H, w_.D, st, w_.occ, w_.params, capi.ADV_SCA_MAC_BFECC) == 0
    dt = float(w_.params.step_time) / w_.params.substeps
    h = float(np.float32(w_.params.voxel_size))
    n = w_.params.substeps
    u, v, w = st["u"], st["v"], st["w"]
    f1 = _py_advect_scalar_mac(T0, u, v, w, w_.occ, n, dt, h)
    f2 = _py_advect_scalar_mac(f1, -u, -v, -w, w_.occ, n, dt, h)
    corrected = T0 * 1.5 - f2 * 0.5
    expect = _py_advect_scalar_mac(corrected, u, v, w, w_.occ, n, dt, h)
    np.testing.assert_array_equal(st["T"], expect)
    assert not np.array_equal(st["T"], T0)


def _py_advect_faces(inp, vel, occ, steps, dt, h):
    """Advect_Velocity_inMAC_outMAC_{u,v,w}_Kernel (Adv3D:233-278 and the v, w
    forms): every face backtraced from its centre through the MAC velocity
    `vel`, the field `inp` (u, v, w) sampled at the last accepted point."""
    D, H, W = occ.shape
    u, v, w = vel
    out = {k: np.empty_like(inp[k]) for k in ("u", "v", "w")}
    starts = {"u": lambda i, j, k: (i, j + 0.5, k + 0.5), "v": lambda i, j, k: (i + 0.5, j, k + 0.5),
              "w": lambda i, j, k: (i + 0.5, j + 0.5, k)}
    shift = {"u": (0.0, 0.5, 0.5), "v": (0.5, 0.0, 0.5), "w": (0.5, 0.5, 0.0)}
    for c in ("u", "v", "w"):
        nz, ny, nx = inp[c].shape
        for k in range(nz):
            for j in range(ny):
                for i in range(nx):
                    last, tri = _py_backtrace_mac(u, v, w, occ, starts[c](i, j, k), steps, dt, h)
                    sx, sy, sz = shift[c]
                    out[c][k, j, i] = tri(inp[c], (last[0] - sx, last[1] - sy, last[2] - sz))
    return out


def _py_apply_open(adv, occ, fld):
    """Apply_Advect_Velocity_Result_Open_{u,v,w}_Kernel (Adv3D:470-576): a face
    takes the advected value when its in-domain cells are free."""
    D, H, W = occ.shape
    free = occ == 0
    for k in range(D):
        for j in range(H):
            for i in range(W + 1):
                if (i == 0 and free[k, j, 0]) or (i == W and free[k, j, W - 1]) or \
                        (0 < i < W and free[k, j, i] and free[k, j, i - 1]):
                    fld["u"][k, j, i] = adv["u"][k, j, i]
    for k in range(D):
        for j in range(H + 1):
            for i in range(W):
                if (j == 0 and free[k, 0, i]) or (j == H and free[k, H - 1, i]) or \
                        (0 < j < H and free[k, j, i] and free[k, j - 1, i]):
                    fld["v"][k, j, i] = adv["v"][k, j, i]
    for k in range(D + 1):
        for j in range(H):
            for i in range(W):
                if (k == 0 and free[0, j, i]) or (k == D and free[D - 1, j, i]) or \
                        (0 < k < D and free[k, j, i] and free[k - 1, j, i]):
                    fld["w"][k, j, i] = adv["w"][k, j, i]


def test_velocity_bfecc_matches_pure_python_restatement(oracle64):
    """cu_Advect_Velocity_inMAC_outMAC_BFECC (Adv3D:1240-1335): forward pass,
    a pass of that result with the negated velocity, u = u*1.5 - back*0.5 in
    place, a forward pass of the corrected field through the original
    velocity, then the open write-back into the corrected field (faces it
    leaves alone keep the corrected value)."""
    w_ = wl.small_case(5, 4, 4, vel_amp=0.4, substeps=2)
    st = {k: np.asarray(v, np.float64).copy() for k, v in w_.state().items()}
    vel0 = {k: st[k].copy() for k in ("u", "v", "w")}
    assert oracle64.advect_velocity(w_.W, w_.H, w_.D, st, w_.occ, w_.params, capi.ADV_VEL_INMAC_OUTMAC_BFECC) == 0
    dt = float(w_.params.step_time) / w_.params.substeps
    h = float(np.float32(w_.params.voxel_size))
    n = w_.params.substeps
    vel = (vel0["u"], vel0["v"], vel0["w"])
    neg = (-vel0["u"], -vel0["v"], -vel0["w"])
    f1 = _py_advect_faces(vel0, vel, w_.occ, n, dt, h)
    f2 = _py_advect_faces(f1, neg, w_.occ, n, dt, h)
    corrected = {k: vel0[k] * 1.5 - f2[k] * 0.5 for k in ("u", "v", "w")}
    f3 = _py_advect_faces(corrected, vel, w_.occ, n, dt, h)
    _py_apply_open(f3, w_.occ, corrected)
    for k in ("u", "v", "w"):
        np.testing.assert_array_equal(st[k], corrected[k], err_msg=k)
        assert not np.array_equal(st[k], vel0[k]), k   # the case moves something


def test_regular_velocity_advection_matches_pure_python_restatement(oracle64):
    """cu_Advect_Velocity_inRegular_outRegular (Adv3D:1061-1101 with the kernel
    at :77-113): cell-centred velocity from the MAC faces, each cell
    backtraced through it and the cell velocity sampled at the last accepted
    point, back to faces (interior faces average their two cells, domain faces
    copy the inner cell), then the open write-back."""
    w_ = wl.small_case(5, 4, 4, vel_amp=0.4, substeps=2)
    st = {k: np.asarray(v, np.float64).copy() for k, v in w_.state().items()}
    u, v, w = (st[k].copy() for k in ("u", "v", "w"))
    assert oracle64.advect_velocity(w_.W, w_.H, w_.D, st, w_.occ, w_.params, capi.ADV_VEL_INREG_OUTREG) == 0
    D, H, W = w_.occ.shape
    dt = float(w_.params.step_time) / w_.params.substeps
    h = float(np.float32(w_.params.voxel_size))
    n = w_.params.substeps
    cx = 0.5 * (u[:, :, :-1] + u[:, :, 1:])
    cy = 0.5 * (v[:, :-1, :] + v[:, 1:, :])
    cz = 0.5 * (w[:-1, :, :] + w[1:, :, :])
    # the MAC helper's tri() applies to any cell field; sample cells at pos - 0.5
    _, tri = _py_backtrace_mac(u, v, w, w_.occ, (0.5, 0.5, 0.5), 0, dt, h)
    cellv = lambda x, y, z: tuple(tri(f, (x - 0.5, y - 0.5, z - 0.5)) for f in (cx, cy, cz))
    out = np.zeros((D, H, W, 3))
    for k in range(D):
        for j in range(H):
            for i in range(W):
                x, y, z = i + 0.5, j + 0.5, k + 0.5
                vx, vy, vz = cellv(x, y, z)
                last = (x, y, z)
                for _ in range(n):
                    if not (0 <= x <= W and 0 <= y <= H and 0 <= z <= D):
                        break
                    if w_.occ[min(max(int(math.floor(z)), 0), D - 1), min(max(int(math.floor(y)), 0), H - 1),
                              min(max(int(math.floor(x)), 0), W - 1)]:
                        break
                    last = (x, y, z)
                    x, y, z = x - (vx * dt) / h, y - (vy * dt) / h, z - (vz * dt) / h
                    vx, vy, vz = cellv(x, y, z)
                out[k, j, i] = cellv(*last)
    fu = np.empty_like(u)
    fu[:, :, 0], fu[:, :, W] = out[:, :, 0, 0], out[:, :, W - 1, 0]
    fu[:, :, 1:W] = 0.5 * (out[:, :, 1:, 0] + out[:, :, :-1, 0])
    fv = np.empty_like(v)
    fv[:, 0, :], fv[:, H, :] = out[:, 0, :, 1], out[:, H - 1, :, 1]
    fv[:, 1:H, :] = 0.5 * (out[:, 1:, :, 1] + out[:, :-1, :, 1])
    fw = np.empty_like(w)
    fw[0], fw[D] = out[0, :, :, 2], out[D - 1, :, :, 2]
    fw[1:D] = 0.5 * (out[1:, :, :, 2] + out[:-1, :, :, 2])
    ref = {"u": u.copy(), "v": v.copy(), "w": w.copy()}
    _py_apply_open({"u": fu, "v": fv, "w": fw}, w_.occ, ref)
    for k in ("u", "v", "w"):
        np.testing.assert_array_equal(st[k], ref[k], err_msg=k)
        assert not np.array_equal(st[k], {"u": u, "v": v, "w": w}[k]), k


def test_force_matches_pure_python_restatement(oracle64):
    """cu_AddForce3D (ZQ_CUDA_AddForce3D.cu:510-556 with the kernels at :11-420):
    cell-centred velocity, vorticity by central differences / (2h) on interior
    cells, the gradient of its magnitude (one-sided at the domain faces,
    normalised when non-zero), force = confine h (N x w) plus buoyancy on y,
    then every face adds dt times the mean of its two free cells' force (one
    cell at a domain face).  Gravity on the density is 0 here (the reference
    has no such term)."""
    W, H, D = 6, 5, 5
    occ = wl.walls_open_top(W, H, D)
    p = wl.smoke_params(W, 1)
    p.confine = 0.3
    p.gravity = 0.0
    rng = np.random.default_rng(8)
    st = {"u": rng.standard_normal((D, H, W + 1)), "v": rng.standard_normal((D, H + 1, W)),
          "w": rng.standard_normal((D + 1, H, W)), "T": rng.random((D, H, W)), "rho": rng.random((D, H, W))}
    u0, v0, w0 = st["u"].copy(), st["v"].copy(), st["w"].copy()
    oracle64.add_force(W, H, D, st, occ, p)
    h, dt = float(np.float32(p.voxel_size)), float(np.float32(p.step_time))
    eps, beta, tamb = float(np.float32(p.confine)), float(np.float32(p.buoyancy)), float(np.float32(p.tamb))
    cu = 0.5 * (u0[:, :, :-1] + u0[:, :, 1:])
    cv = 0.5 * (v0[:, :-1, :] + v0[:, 1:, :])
    cw = 0.5 * (w0[:-1, :, :] + w0[1:, :, :])
    vort = np.zeros((D, H, W, 3))
    vs = np.zeros((D, H, W))
    for k in range(1, D - 1):
        for j in range(1, H - 1):
            for i in range(1, W - 1):
                a = (cw[k, j + 1, i] - cw[k, j - 1, i] - cv[k + 1, j, i] + cv[k - 1, j, i]) / (2 * h)
                b = (cu[k + 1, j, i] - cu[k - 1, j, i] - cw[k, j, i + 1] + cw[k, j, i - 1]) / (2 * h)
                c = (cv[k, j, i + 1] - cv[k, j, i - 1] - cu[k, j + 1, i] + cu[k, j - 1, i]) / (2 * h)
                vort[k, j, i] = (a, b, c)
                vs[k, j, i] = math.sqrt(a * a + b * b + c * c)
    force = np.zeros((D, H, W, 3))
    for k in range(D):
        for j in range(H):
            for i in range(W):
                def g(axis):
                    # d|w|/d(axis): one-sided at the domain faces, central inside
                    n, pos = (W, H, D)[axis], (i, j, k)[axis]

                    def at(q):
                        t = [i, j, k]
                        t[axis] = q
                        return vs[t[2], t[1], t[0]]
                    if pos == 0:
                        return at(1) - at(0)
                    if pos == n - 1:
                        return at(n - 1) - at(n - 2)
                    return 0.5 * (at(pos + 1) - at(pos - 1))
                gx, gy, gz = g(0), g(1), g(2)
                ln = math.sqrt(gx * gx + gy * gy + gz * gz)
                if ln != 0:
                    gx, gy, gz = gx / ln, gy / ln, gz / ln
                wx, wy, wz = vort[k, j, i]
                fx = eps * h * (gy * wz - gz * wy)
                fy = eps * h * (gz * wx - gx * wz)
                fz = eps * h * (gx * wy - gy * wx)
                fy = fy + beta * (st["T"][k, j, i] - tamb)
                force[k, j, i] = (fx, fy, fz)
    free = occ == 0
    eu, ev, ew = u0.copy(), v0.copy(), w0.copy()
    for k in range(D):
        for j in range(H):
            for i in range(W + 1):
                if i == 0:
                    if free[k, j, 0]:
                        eu[k, j, i] += dt * force[k, j, 0, 0]
                elif i == W:
                    if free[k, j, W - 1]:
                        eu[k, j, i] += dt * force[k, j, W - 1, 0]
                elif free[k, j, i] and free[k, j, i - 1]:
                    eu[k, j, i] += dt * 0.5 * (force[k, j, i, 0] + force[k, j, i - 1, 0])
    for k in range(D):
        for j in range(H + 1):
            for i in range(W):
                if j == 0:
                    if free[k, 0, i]:
                        ev[k, j, i] += dt * force[k, 0, i, 1]
                elif j == H:
                    if free[k, H - 1, i]:
                        ev[k, j, i] += dt * force[k, H - 1, i, 1]
                elif free[k, j, i] and free[k, j - 1, i]:
                    ev[k, j, i] += dt * 0.5 * (force[k, j, i, 1] + force[k, j - 1, i, 1])
    for k in range(D + 1):
        for j in range(H):
            for i in range(W):
                if k == 0:
                    if free[0, j, i]:
                        ew[k, j, i] += dt * force[0, j, i, 2]
                elif k == D:
                    if free[D - 1, j, i]:
                        ew[k, j, i] += dt * force[D - 1, j, i, 2]
                elif free[k, j, i] and free[k - 1, j, i]:
                    ew[k, j, i] += dt * 0.5 * (force[k, j, i, 2] + force[k - 1, j, i, 2])
    for name, got, exp in (("u", st["u"], eu), ("v", st["v"], ev), ("w", st["w"], ew)):
        np.testing.assert_array_equal(got, exp, err_msg=name)
        assert not np.array_equal(got, {"u": u0, "v": v0, "w": w0}[name]), name


def test_regular_velocity_scalar_advection_matches_pure_python_restatement(oracle64):
    """cu_Advect_Scalar_Regular_Velocity (Adv3D:380-418 and :1456-1505): the
    MAC velocity to cell centres, each cell backtraced through it from its
    centre, temperature and density sampled at the last accepted point."""
    w_ = wl.small_case(6, 5, 4, vel_amp=0.4, substeps=3)
    st = {k: np.asarray(v, np.float64).copy() for k, v in w_.state().items()}
    T0, R0 = st["T"].copy(), st["rho"].copy()
    u, v, w = st["u"], st["v"], st["w"]
    assert oracle64.advect_scalar(w_.W, w_.H, w_.D, st, w_.occ, w_.params, capi.ADV_SCA_REG) == 0
    D, H, W = w_.occ.shape
    dt = float(w_.params.step_time) / w_.params.substeps
    h = float(np.float32(w_.params.voxel_size))
    cx = 0.5 * (u[:, :, :-1] + u[:, :, 1:])
    cy = 0.5 * (v[:, :-1, :] + v[:, 1:, :])
    cz = 0.5 * (w[:-1, :, :] + w[1:, :, :])
    _, tri = _py_backtrace_mac(u, v, w, w_.occ, (0.5, 0.5, 0.5), 0, dt, h)
    cellv = lambda x, y, z: tuple(tri(f, (x - 0.5, y - 0.5, z - 0.5)) for f in (cx, cy, cz))
    for k in range(D):
        for j in range(H):
            for i in range(W):
                x, y, z = i + 0.5, j + 0.5, k + 0.5
                vx, vy, vz = cellv(x, y, z)
                last = (x, y, z)
                for _ in range(w_.params.substeps):
                    if not (0 <= x <= W and 0 <= y <= H and 0 <= z <= D):
                        break
                    if w_.occ[min(max(int(math.floor(z)), 0), D - 1), min(max(int(math.floor(y)), 0), H - 1),
                              min(max(int(math.floor(x)), 0), W - 1)]:
                        break
                    last = (x, y, z)
                    x, y, z = x - (vx * dt) / h, y - (vy * dt) / h, z - (vz * dt) / h
                    vx, vy, vz = cellv(x, y, z)
                g = (last[0] - 0.5, last[1] - 0.5, last[2] - 0.5)
                assert st["T"][k, j, i] == tri(T0, g), (i, j, k)
                assert st["rho"][k, j, i] == tri(R0, g), (i, j, k)
    assert not np.array_equal(st["T"], T0)


def test_regular_in_mac_out_velocity_advection_matches_pure_python_restatement(oracle64):
    """cu_Advect_Velocity_inRegular_outMAC (Adv3D:1337-1380 with the kernels at
    :116-230): every face backtraced from its centre through the cell-centred
    velocity, the face's own component of that velocity sampled at the last
    accepted point, then the open write-back."""
    w_ = wl.small_case(5, 4, 4, vel_amp=0.4, substeps=2)
    st = {k: np.asarray(v, np.float64).copy() for k, v in w_.state().items()}
    u, v, w = (st[k].copy() for k in ("u", "v", "w"))
    assert oracle64.advect_velocity(w_.W, w_.H, w_.D, st, w_.occ, w_.params, capi.ADV_VEL_INREG_OUTMAC) == 0
    D, H, W = w_.occ.shape
    dt = float(w_.params.step_time) / w_.params.substeps
    h = float(np.float32(w_.params.voxel_size))
    n = w_.params.substeps
    cx = 0.5 * (u[:, :, :-1] + u[:, :, 1:])
    cy = 0.5 * (v[:, :-1, :] + v[:, 1:, :])
    cz = 0.5 * (w[:-1, :, :] + w[1:, :, :])
    _, tri = _py_backtrace_mac(u, v, w, w_.occ, (0.5, 0.5, 0.5), 0, dt, h)
    cellv = lambda x, y, z: tuple(tri(f, (x - 0.5, y - 0.5, z - 0.5)) for f in (cx, cy, cz))

    def trace(x, y, z):
        vx, vy, vz = cellv(x, y, z)
        last = (x, y, z)
        for _ in range(n):
            if not (0 <= x <= W and 0 <= y <= H and 0 <= z <= D):
                break
            if w_.occ[min(max(int(math.floor(z)), 0), D - 1), min(max(int(math.floor(y)), 0), H - 1),
                      min(max(int(math.floor(x)), 0), W - 1)]:
                break
            last = (x, y, z)
            x, y, z = x - (vx * dt) / h, y - (vy * dt) / h, z - (vz * dt) / h
            vx, vy, vz = cellv(x, y, z)
        return cellv(*last)

    adv = {"u": np.empty_like(u), "v": np.empty_like(v), "w": np.empty_like(w)}
    for k in range(D):
        for j in range(H):
            for i in range(W + 1):
                adv["u"][k, j, i] = trace(i, j + 0.5, k + 0.5)[0]
    for k in range(D):
        for j in range(H + 1):
            for i in range(W):
                adv["v"][k, j, i] = trace(i + 0.5, j, k + 0.5)[1]
    for k in range(D + 1):
        for j in range(H):
            for i in range(W):
                adv["w"][k, j, i] = trace(i + 0.5, j + 0.5, k)[2]
    ref = {"u": u.copy(), "v": v.copy(), "w": w.copy()}
    _py_apply_open(adv, w_.occ, ref)
    for k in ("u", "v", "w"):
        np.testing.assert_array_equal(st[k], ref[k], err_msg=k)
        assert not np.array_equal(st[k], {"u": u, "v": v, "w": w}[k]), k


def test_mac_velocity_advection_closed_writeback_matches_restatement(oracle64):
    """cu_Advect_Velocity_inMAC_outMAC with the closed write-back
    (Apply_Advect_Velocity_Result_Closed_*, Adv3D:577-650): only interior faces
    between two free cells take the advected value; domain faces keep theirs."""
    w_ = wl.small_case(5, 4, 4, vel_amp=0.4, substeps=2)
    st = {k: np.asarray(v, np.float64).copy() for k, v in w_.state().items()}
    vel0 = {k: st[k].copy() for k in ("u", "v", "w")}
    assert oracle64.advect_velocity(w_.W, w_.H, w_.D, st, w_.occ, w_.params, capi.ADV_VEL_INMAC_OUTMAC,
                                    is_open=False) == 0
    D, H, W = w_.occ.shape
    dt = float(w_.params.step_time) / w_.params.substeps
    h = float(np.float32(w_.params.voxel_size))
    adv = _py_advect_faces(vel0, (vel0["u"], vel0["v"], vel0["w"]), w_.occ, w_.params.substeps, dt, h)
    free = w_.occ == 0
    ref = {k: vel0[k].copy() for k in ("u", "v", "w")}
    ref["u"][:, :, 1:W] = np.where(free[:, :, 1:] & free[:, :, :-1], adv["u"][:, :, 1:W], ref["u"][:, :, 1:W])
    ref["v"][:, 1:H, :] = np.where(free[:, 1:, :] & free[:, :-1, :], adv["v"][:, 1:H, :], ref["v"][:, 1:H, :])
    ref["w"][1:D] = np.where(free[1:] & free[:-1], adv["w"][1:D], ref["w"][1:D])
    for k in ("u", "v", "w"):
        np.testing.assert_array_equal(st[k], ref[k], err_msg=k)


def _py_advect_scalar_reg(phi, cx, cy, cz, occ, steps, dt, h, tri):
    """One pass of Advect_Scalar_Regular_Velocity_Kernel over a cell field with
    the cell-centred velocity (cx, cy, cz)."""
    D, H, W = occ.shape
    cellv = lambda x, y, z: tuple(tri(f, (x - 0.5, y - 0.5, z - 0.5)) for f in (cx, cy, cz))
    out = np.empty_like(phi)
    for k in range(D):
        for j in range(H):
            for i in range(W):
                x, y, z = i + 0.5, j + 0.5, k + 0.5
                vx, vy, vz = cellv(x, y, z)
                last = (x, y, z)
                for _ in range(steps):
                    if not (0 <= x <= W and 0 <= y <= H and 0 <= z <= D):
                        break
                    if occ[min(max(int(math.floor(z)), 0), D - 1), min(max(int(math.floor(y)), 0), H - 1),
                           min(max(int(math.floor(x)), 0), W - 1)]:
                        break
                    last = (x, y, z)
                    x, y, z = x - (vx * dt) / h, y - (vy * dt) / h, z - (vz * dt) / h
                    vx, vy, vz = cellv(x, y, z)
                out[k, j, i] = tri(phi, (last[0] - 0.5, last[1] - 0.5, last[2] - 0.5))
    return out


def test_regular_scalar_bfecc_matches_pure_python_restatement(oracle64):
    """cu_Advect_Scalar_Regular_Velocity_BFECC (Adv3D:1507-1554): forward with
    the cell-centred velocity, back with it negated
    (Velocity_Negative_4channels), input = input*1.5 - back*0.5, forward."""
    w_ = wl.small_case(6, 5, 4, vel_amp=0.4, substeps=2)
    st = {k: np.asarray(v, np.float64).copy() for k, v in w_.state().items()}
    T0 = st["T"].copy()
    u, v, w = st["u"], st["v"], st["w"]
    assert oracle64.advect_scalar(w_.W, w_.H, w_.D, st, w_.occ, w_.params, capi.ADV_SCA_REG_BFECC) == 0
    dt = float(w_.params.step_time) / w_.params.substeps
    h = float(np.float32(w_.params.voxel_size))
    n = w_.params.substeps
    cx = 0.5 * (u[:, :, :-1] + u[:, :, 1:])
    cy = 0.5 * (v[:, :-1, :] + v[:, 1:, :])
    cz = 0.5 * (w[:-1, :, :] + w[1:, :, :])
    _, tri = _py_backtrace_mac(u, v, w, w_.occ, (0.5, 0.5, 0.5), 0, dt, h)
    f1 = _py_advect_scalar_reg(T0, cx, cy, cz, w_.occ, n, dt, h, tri)
    f2 = _py_advect_scalar_reg(f1, -cx, -cy, -cz, w_.occ, n, dt, h, tri)
    corrected = T0 * 1.5 - f2 * 0.5
    expect = _py_advect_scalar_reg(corrected, cx, cy, cz, w_.occ, n, dt, h, tri)
    np.testing.assert_array_equal(st["T"], expect)
    assert not np.array_equal(st["T"], T0)


def test_regular_velocity_bfecc_matches_pure_python_restatement(oracle64):
    """cu_Advect_Velocity_inRegular_outRegular_BFECC (Adv3D:1103-1176): on the
    cell-centred velocity c, c1 = A(c; c), c2 = A(c1; -c), c' = c*1.5 - c2*0.5
    (Input_Increment_4channels_Kernel), c3 = A(c'; c), back to faces and the
    open write-back into the untouched MAC fields."""
    w_ = wl.small_case(5, 4, 4, vel_amp=0.4, substeps=2)
    st = {k: np.asarray(v, np.float64).copy() for k, v in w_.state().items()}
    u, v, w = (st[k].copy() for k in ("u", "v", "w"))
    assert oracle64.advect_velocity(w_.W, w_.H, w_.D, st, w_.occ, w_.params, capi.ADV_VEL_INREG_OUTREG_BFECC) == 0
    D, H, W = w_.occ.shape
    dt = float(w_.params.step_time) / w_.params.substeps
    h = float(np.float32(w_.params.voxel_size))
    n = w_.params.substeps
    c = [0.5 * (u[:, :, :-1] + u[:, :, 1:]), 0.5 * (v[:, :-1, :] + v[:, 1:, :]), 0.5 * (w[:-1, :, :] + w[1:, :, :])]
    _, tri = _py_backtrace_mac(u, v, w, w_.occ, (0.5, 0.5, 0.5), 0, dt, h)
    adv = lambda fields, vel: [_py_advect_scalar_reg(f, *vel, w_.occ, n, dt, h, tri) for f in fields]
    c1 = adv(c, c)
    c2 = adv(c1, [-a for a in c])
    cc = [a * 1.5 - b * 0.5 for a, b in zip(c, c2)]
    c3 = adv(cc, c)
    fu = np.empty_like(u)
    fu[:, :, 0], fu[:, :, W] = c3[0][:, :, 0], c3[0][:, :, W - 1]
    fu[:, :, 1:W] = 0.5 * (c3[0][:, :, 1:] + c3[0][:, :, :-1])
    fv = np.empty_like(v)
    fv[:, 0, :], fv[:, H, :] = c3[1][:, 0, :], c3[1][:, H - 1, :]
    fv[:, 1:H, :] = 0.5 * (c3[1][:, 1:, :] + c3[1][:, :-1, :])
    fw = np.empty_like(w)
    fw[0], fw[D] = c3[2][0], c3[2][D - 1]
    fw[1:D] = 0.5 * (c3[2][1:] + c3[2][:-1])
    ref = {"u": u.copy(), "v": v.copy(), "w": w.copy()}
    _py_apply_open({"u": fu, "v": fv, "w": fw}, w_.occ, ref)
    for k in ("u", "v", "w"):
        np.testing.assert_array_equal(st[k], ref[k], err_msg=k)


def test_regular_in_mac_out_velocity_bfecc_matches_pure_python_restatement(oracle64):
    """cu_Advect_Velocity_inRegular_outMAC_BFECC (Adv3D:1389-1466): faces
    out1 = A(c; c) traced through the cell velocity c, out2 = A(reg(out1); -c),
    then the input c*1.5 - reg(out2)*0.5 (the velocity texture is copied
    before Input_Increment_4channels, so the trace stays on c), out3 =
    A(that; c) and the open write-back into the untouched MAC fields."""
    w_ = wl.small_case(5, 4, 4, vel_amp=0.4, substeps=2)
    st = {k: np.asarray(v, np.float64).copy() for k, v in w_.state().items()}
    u, v, w = (st[k].copy() for k in ("u", "v", "w"))
    assert oracle64.advect_velocity(w_.W, w_.H, w_.D, st, w_.occ, w_.params, capi.ADV_VEL_INREG_OUTMAC_BFECC) == 0
    D, H, W = w_.occ.shape
    dt = float(w_.params.step_time) / w_.params.substeps
    h = float(np.float32(w_.params.voxel_size))
    n = w_.params.substeps
    reg = lambda fu, fv, fw: [0.5 * (fu[:, :, :-1] + fu[:, :, 1:]), 0.5 * (fv[:, :-1, :] + fv[:, 1:, :]),
                              0.5 * (fw[:-1, :, :] + fw[1:, :, :])]
    c = reg(u, v, w)
    _, tri = _py_backtrace_mac(u, v, w, w_.occ, (0.5, 0.5, 0.5), 0, dt, h)
    at = lambda fields, x, y, z: tuple(tri(f, (x - 0.5, y - 0.5, z - 0.5)) for f in fields)

    def trace(vel, inp, x, y, z, comp):
        vx, vy, vz = at(vel, x, y, z)
        last = (x, y, z)
        for _ in range(n):
            if not (0 <= x <= W and 0 <= y <= H and 0 <= z <= D):
                break
            if w_.occ[min(max(int(math.floor(z)), 0), D - 1), min(max(int(math.floor(y)), 0), H - 1),
                      min(max(int(math.floor(x)), 0), W - 1)]:
                break
            last = (x, y, z)
            x, y, z = x - (vx * dt) / h, y - (vy * dt) / h, z - (vz * dt) / h
            vx, vy, vz = at(vel, x, y, z)
        return tri(inp[comp], (last[0] - 0.5, last[1] - 0.5, last[2] - 0.5))

    def faces(vel, inp):
        fu, fv, fw = np.empty_like(u), np.empty_like(v), np.empty_like(w)
        for k in range(D):
            for j in range(H):
                for i in range(W + 1):
                    fu[k, j, i] = trace(vel, inp, i, j + 0.5, k + 0.5, 0)
        for k in range(D):
            for j in range(H + 1):
                for i in range(W):
                    fv[k, j, i] = trace(vel, inp, i + 0.5, j, k + 0.5, 1)
        for k in range(D + 1):
            for j in range(H):
                for i in range(W):
                    fw[k, j, i] = trace(vel, inp, i + 0.5, j + 0.5, k, 2)
        return fu, fv, fw

    out1 = faces(c, c)
    out2 = faces([-a for a in c], reg(*out1))
    cc = [a * 1.5 - b * 0.5 for a, b in zip(c, reg(*out2))]
    out3 = faces(c, cc)
    ref = {"u": u.copy(), "v": v.copy(), "w": w.copy()}
    _py_apply_open(dict(zip(("u", "v", "w"), out3)), w_.occ, ref)
    for k in ("u", "v", "w"):
        np.testing.assert_array_equal(st[k], ref[k], err_msg=k)


def test_attenuation_matches_pure_python_restatement(oracle64):
    """Atten_{u,v,w}_Kernel and Atten_temperature_density_Kernel
    (ZQ_CUDA_Attenuation3D.cu:8-116): a face is scaled by the velocity factor
    when both of its cells are free (a domain face: its one inner cell), and
    every cell's temperature and density by their factors, occupied or not."""
    w_ = wl.small_case(5, 4, 4, vel_amp=0.4, substeps=2)
    p = w_.params
    p.vel_atten, p.temp_atten, p.dens_atten = 0.75, 0.5, 0.25
    st = {k: np.asarray(v, np.float64).copy() for k, v in w_.state().items()}
    ref = {k: a.copy() for k, a in st.items()}
    oracle64.attenuate(w_.W, w_.H, w_.D, st, w_.occ, p)
    occ = w_.occ.astype(bool)
    D, H, W = occ.shape
    for k in range(D):
        for j in range(H):
            for i in range(W + 1):
                if not (i > 0 and occ[k, j, i - 1]) and not (i < W and occ[k, j, i]):
                    ref["u"][k, j, i] *= 0.75
    for k in range(D):
        for j in range(H + 1):
            for i in range(W):
                if not (j > 0 and occ[k, j - 1, i]) and not (j < H and occ[k, j, i]):
                    ref["v"][k, j, i] *= 0.75
    for k in range(D + 1):
        for j in range(H):
            for i in range(W):
                if not (k > 0 and occ[k - 1, j, i]) and not (k < D and occ[k, j, i]):
                    ref["w"][k, j, i] *= 0.75
    ref["T"] *= 0.5
    ref["rho"] *= 0.25
    assert occ.any() and not occ.all()
    for k in ref:
        np.testing.assert_array_equal(st[k], ref[k], err_msg=k)


@pytest.mark.parametrize("vmode,smode", [(capi.ADV_VEL_INMAC_OUTMAC, capi.ADV_SCA_MAC),
                                         (capi.ADV_VEL_INREG_OUTREG_BFECC, capi.ADV_SCA_REG_BFECC)])
def test_step_is_the_reference_stage_order(oracle64, vmode, smode):
    """ZQ_SmokeSimulation3D::UpdateOneFrame (ZQ_SmokeSimulation3D.cpp:156-243):
    force, attenuation, velocity advection, projection, scalar advection,
    reinjection.  The oracle's step must equal its stages run in that order."""
    w_ = wl.small_case(6, 5, 4, vel_amp=0.4, substeps=2)
    p = w_.params
    p.vel_atten, p.temp_atten, p.dens_atten = 0.9, 0.8, 0.7
    p.adv_vel_mode, p.adv_sca_mode = vmode, smode
    st = {k: np.asarray(v, np.float64).copy() for k, v in w_.state().items()}
    ref = {k: a.copy() for k, a in st.items()}
    rc, _ = oracle64.step(w_.W, w_.H, w_.D, st, w_.occ, p, 1)
    assert rc == 0
    oracle64.add_force(w_.W, w_.H, w_.D, ref, w_.occ, p)
    oracle64.attenuate(w_.W, w_.H, w_.D, ref, w_.occ, p)
    assert oracle64.advect_velocity(w_.W, w_.H, w_.D, ref, w_.occ, p, vmode) == 0
    oracle64.project(w_.W, w_.H, w_.D, ref, w_.occ, p)
    assert oracle64.advect_scalar(w_.W, w_.H, w_.D, ref, w_.occ, p, smode) == 0
    oracle64.reinject(w_.W, w_.H, w_.D, ref, p)
    for k in ("u", "v", "w", "T", "rho"):
        np.testing.assert_array_equal(st[k], ref[k], err_msg=k)
    # a different order gives a different state (the pin is not vacuous)
    alt = {k: np.asarray(v, np.float64).copy() for k, v in w_.state().items()}
    oracle64.attenuate(w_.W, w_.H, w_.D, alt, w_.occ, p)
    oracle64.add_force(w_.W, w_.H, w_.D, alt, w_.occ, p)
    oracle64.advect_velocity(w_.W, w_.H, w_.D, alt, w_.occ, p, vmode)
    oracle64.project(w_.W, w_.H, w_.D, alt, w_.occ, p)
    oracle64.advect_scalar(w_.W, w_.H, w_.D, alt, w_.occ, p, smode)
    oracle64.reinject(w_.W, w_.H, w_.D, alt, p)
    assert not np.array_equal(alt["v"], st["v"])
