"""Known answers of the oracle's coarse-grid projection (no GPU).

ZQS_SOLVER_COARSE_OPEN restates ZQ_TotalProjection3D for the coarse SOR
solvers (Utils3D:3688-3794): face-ratio SOR on the grid coarsened by s, the
correction mapped back to the fine faces, then an exact projection inside
every s^3 block (dense matrix of ZQ_InitSubMatPoisson3D for blocks without
obstacles, a least-squares solve for the others).
"""
import numpy as np
import pytest

from conftest import rel_l2
from zq_smokesimulation_gb300 import capi
from zq_smokesimulation_gb300 import workloads as wl


def block_faces(s):
    """Block face index helpers in the matrix column order (u, v, w)."""
    nu = s * s * (s + 1)
    uix = lambda i, j, k: (k * s + j) * (s + 1) + i
    vix = lambda i, j, k: nu + (k * (s + 1) + j) * s + i
    wix = lambda i, j, k: 2 * nu + (k * s + j) * s + i
    rows = ([uix(i, j, k) for k in range(s) for j in range(s) for i in range(1, s)] +
            [vix(i, j, k) for k in range(s) for j in range(1, s) for i in range(s)] +
            [wix(i, j, k) for k in range(1, s) for j in range(s) for i in range(s)])
    return uix, vix, wix, rows


def block_div(x, s):
    uix, vix, wix, _ = block_faces(s)
    return np.array([[[(x[uix(i + 1, j, k)] - x[uix(i, j, k)]) + (x[vix(i, j + 1, k)] - x[vix(i, j, k)]) +
                       (x[wix(i, j, k + 1)] - x[wix(i, j, k)]) for i in range(s)] for j in range(s)]
                     for k in range(s)])


@pytest.mark.parametrize("s", [2, 3, 4])
def test_submatrix_keeps_uniform_flow(oracle32, s):
    M = oracle32.submatrix(s).astype(np.float64)
    uix, vix, wix, rows = block_faces(s)
    x = np.zeros(M.shape[1])
    nu = s * s * (s + 1)
    x[:nu], x[nu:2 * nu], x[2 * nu:] = 0.3, -0.7, 1.1
    np.testing.assert_allclose(M @ x, x[rows], rtol=0, atol=1e-6)


@pytest.mark.parametrize("s", [2, 4])
def test_submatrix_leaves_the_mean_divergence(oracle32, s):
    """The block least-squares projection leaves div = mean(div) in every cell
    (the residual of the pinned Neumann problem is the constant component)."""
    M = oracle32.submatrix(s).astype(np.float64)
    _, _, _, rows = block_faces(s)
    x = np.random.default_rng(3).standard_normal(M.shape[1])
    y = x.copy()
    y[rows] = M @ x
    d0, d1 = block_div(x, s), block_div(y, s)
    np.testing.assert_allclose(d1, np.full_like(d1, d0.mean()), atol=2e-5 * np.abs(d0).max())


@pytest.mark.parametrize("s", [2, 3, 4])
def test_submatrix_equals_the_svd_pseudo_inverse_form(oracle32, s):
    """ZQ_InitSubMatPoisson3D (Utils3D:1151-1391) forms the block matrix with
    an SVD pseudo-inverse (ZQ_SVD::Invert): with L the block's Neumann
    Laplacian, P = L without cell 0's column, V the cell divergence over the
    block faces, pressures p = [0; P+ V x] and the interior faces x - (p_b - p_a).
    The oracle builds P+ by Cholesky on the normal equations; numpy's pinv (an
    SVD) gives the same matrix to rounding."""
    n, nf = s ** 3, 3 * s * s * (s + 1)
    uix, vix, wix, rows = block_faces(s)
    cell = lambda i, j, k: (k * s + j) * s + i
    L = np.zeros((n, n))
    V = np.zeros((n, nf))
    for k in range(s):
        for j in range(s):
            for i in range(s):
                c = cell(i, j, k)
                for di, dj, dk in ((-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)):
                    a, b, e = i + di, j + dj, k + dk
                    if 0 <= a < s and 0 <= b < s and 0 <= e < s:
                        L[c, cell(a, b, e)] = 1.0
                        L[c, c] -= 1.0
                V[c, uix(i + 1, j, k)] += 1.0
                V[c, uix(i, j, k)] -= 1.0
                V[c, vix(i, j + 1, k)] += 1.0
                V[c, vix(i, j, k)] -= 1.0
                V[c, wix(i, j, k + 1)] += 1.0
                V[c, wix(i, j, k)] -= 1.0
    pres = np.vstack([np.zeros((1, nf)), np.linalg.pinv(L[:, 1:]) @ V])   # n x nf, cell 0 pinned to 0
    ref = []
    for k in range(s):
        for j in range(s):
            for i in range(1, s):
                ref.append(np.eye(nf)[uix(i, j, k)] - (pres[cell(i, j, k)] - pres[cell(i - 1, j, k)]))
    for k in range(s):
        for j in range(1, s):
            for i in range(s):
                ref.append(np.eye(nf)[vix(i, j, k)] - (pres[cell(i, j, k)] - pres[cell(i, j - 1, k)]))
    for k in range(1, s):
        for j in range(s):
            for i in range(s):
                ref.append(np.eye(nf)[wix(i, j, k)] - (pres[cell(i, j, k)] - pres[cell(i, j, k - 1)]))
    ref = np.array(ref)
    M = oracle32.submatrix(s).astype(np.float64)
    assert M.shape == ref.shape
    np.testing.assert_allclose(M, ref, rtol=0, atol=2e-6 * np.abs(ref).max())


def coarse_case(W, H, D, s, K, seed=5, walls=True, omega=1.5):
    occ = wl.walls_open_top(W, H, D) if walls else np.zeros((D, H, W), np.uint8)
    p = wl.smoke_params(W, K, omega=omega, solver=capi.SOLVER_COARSE_OPEN)
    p.sub_size = s
    u, v, w = wl.initial_velocity(occ, seed, amp=1.0)
    return occ, p, {"u": u.copy(), "v": v.copy(), "w": w.copy()}


def max_div(st, occ):
    u, v, w = st["u"].astype(np.float64), st["v"].astype(np.float64), st["w"].astype(np.float64)
    d = (u[:, :, 1:] - u[:, :, :-1]) + (v[:, 1:, :] - v[:, :-1, :]) + (w[1:, :, :] - w[:-1, :, :])
    return float(np.abs(d[occ == 0]).max())


def test_coarse_s1_matches_the_fine_open_sor(oracle32):
    """With s = 1 the coarse grid is the fine grid (ratios 0/1) and the same
    SOR runs; only the correction is formed as u + ((u - g) - u)."""
    occ, p, st = coarse_case(12, 10, 9, 1, K=30)
    ref = {k: a.copy() for k, a in st.items()}
    p_open = p.copy()
    p_open.solver = capi.SOLVER_OPEN
    oracle32.project(12, 10, 9, ref, occ, p_open)
    assert oracle32.project_coarse(12, 10, 9, st, occ, p) == 0
    for k in ("u", "v", "w"):
        assert rel_l2(st[k], ref[k]) < 1e-6, k


@pytest.mark.parametrize("walls", [False, True])
def test_coarse_projection_removes_divergence(oracle32, walls):
    """Without obstacles the result is divergence-free to rounding.  With walls
    the coarse system of ZQ_InitMatOpenPoisson3D gives every domain face weight
    1 whatever its un-occupancy ratio, while the correction moves only the free
    fine faces, so blocks at the walls keep a residual (a property of the
    formulation, as restated)."""
    occ, p, st = coarse_case(16, 16, 16, 4, K=400, walls=walls)
    before = max_div(st, occ)
    assert oracle32.project_coarse(16, 16, 16, st, occ, p) == 0
    after = max_div(st, occ)
    assert after < (0.05 if walls else 1e-4) * before, (before, after)


def test_coarse_rejects_sizes_not_divisible(oracle32):
    occ, p, st = coarse_case(12, 12, 12, 4, K=2)
    p.sub_size = 5
    assert oracle32.project_coarse(12, 12, 12, st, occ, p) == capi.ZQS_EINVAL


def _py_block_projection(u, v, w, occ, s):
    """ZQ_SubProjection3D / ZQ_SolveSubGrid3D restated with numpy: in every
    s^3 block, the pressure of the least-squares Poisson problem of its free
    cells (weight 1 between free in-block neighbours, right-hand side the
    cell divergence over the block's faces; numpy's lstsq gives the
    minimum-norm least-squares solution, as the reference's SVD / PCG do), then
    u_face -= p_b - p_a on the faces between two free cells of the block."""
    D, H, W = occ.shape
    u, v, w = u.copy(), v.copy(), w.copy()
    for bk in range(D // s):
        for bj in range(H // s):
            for bi in range(W // s):
                cells = [(i, j, k) for k in range(bk * s, bk * s + s) for j in range(bj * s, bj * s + s)
                         for i in range(bi * s, bi * s + s) if not occ[k, j, i]]
                if not cells:
                    continue
                ix = {c: n for n, c in enumerate(cells)}
                L = np.zeros((len(cells), len(cells)))
                b = np.zeros(len(cells))
                inb = lambda i, j, k: bi * s <= i < bi * s + s and bj * s <= j < bj * s + s and bk * s <= k < bk * s + s
                for (i, j, k), n in ix.items():
                    b[n] = (u[k, j, i + 1] - u[k, j, i]) + (v[k, j + 1, i] - v[k, j, i]) + (w[k + 1, j, i] - w[k, j, i])
                    for di, dj, dk in ((-1, 0, 0), (1, 0, 0), (0, -1, 0), (0, 1, 0), (0, 0, -1), (0, 0, 1)):
                        nb = (i + di, j + dj, k + dk)
                        if inb(*nb) and nb in ix:
                            L[n, ix[nb]] += 1.0
                            L[n, n] -= 1.0
                # lstsq cuts the zero singular values (pinv without a cutoff
                # would invert the rounding noise of the singular direction)
                p = np.linalg.lstsq(L, b, rcond=None)[0]
                for (i, j, k), n in ix.items():
                    if (i - 1, j, k) in ix and inb(i - 1, j, k):
                        u[k, j, i] -= p[n] - p[ix[(i - 1, j, k)]]
                    if (i, j - 1, k) in ix and inb(i, j - 1, k):
                        v[k, j, i] -= p[n] - p[ix[(i, j - 1, k)]]
                    if (i, j, k - 1) in ix and inb(i, j, k - 1):
                        w[k, j, i] -= p[n] - p[ix[(i, j, k - 1)]]
    return u, v, w


@pytest.mark.parametrize("s", [2, 4])
def test_block_projection_matches_least_squares_restatement(oracle64, s):
    """With no coarse iterations (K = 0) the coarse correction is exactly zero
    and the projection is the block step alone: dense-matrix blocks and
    obstacle blocks against the numpy least-squares restatement."""
    W, H, D = 8, 8, 8
    occ = wl.walls_open_top(W, H, D)
    wl.add_box(occ, 3, 4, 2, 5, 3, 3)
    p = wl.smoke_params(W, 0, omega=1.5, solver=capi.SOLVER_COARSE_OPEN)
    p.sub_size = s
    u, v, w = wl.initial_velocity(occ, 4, amp=1.0)
    st = {"u": np.asarray(u, np.float64).copy(), "v": np.asarray(v, np.float64).copy(),
          "w": np.asarray(w, np.float64).copy()}
    assert oracle64.project_coarse(W, H, D, st, occ, p) == 0
    eu, ev, ew = _py_block_projection(np.asarray(u, np.float64), np.asarray(v, np.float64),
                                      np.asarray(w, np.float64), occ, s)
    scale = max(np.abs(eu).max(), np.abs(ev).max(), np.abs(ew).max())
    for name, got, exp in (("u", st["u"], eu), ("v", st["v"], ev), ("w", st["w"], ew)):
        # the dense blocks use the block matrix rounded to float, as the reference stores it
        np.testing.assert_allclose(got, exp, rtol=0, atol=2e-6 * scale, err_msg=name)
    assert not np.allclose(st["u"], u)


def _py_coarse_correction(u, v, w, occ, s, K, omega):
    """The coarse stages of ZQ_TotalProjection3D restated with numpy loops:
    face un-occupancy ratios and coarse occupancy (ZQ_InitCoarseGrid3D,
    Utils3D:1666-1888), fine faces averaged onto coarse faces
    (ZQ_MapFine2Coarse3D, :2170-2258), K red-black SOR iterations of the
    face-ratio system (domain faces weight 1, p = 0 outside), the correction
    (u - g) - u on faces with ratio > 0, added to the fine faces on coarse
    faces whose cells are free (ZQ_MapCoarse2Fine3D, :3172-3296)."""
    D, H, W = occ.shape
    cD, cH, cW = D // s, H // s, W // s
    ru, rv, rw = np.zeros((cD, cH, cW + 1)), np.zeros((cD, cH + 1, cW)), np.zeros((cD + 1, cH, cW))
    for k in range(cD):
        for j in range(cH):
            for i in range(cW + 1):
                n = 0
                for sk in range(s):
                    for sj in range(s):
                        z, y, x = k * s + sk, j * s + sj, i * s
                        n += bool(occ[z, y, 0]) if i == 0 else bool(occ[z, y, W - 1]) if i == cW else \
                            bool(occ[z, y, x] or occ[z, y, x - 1])
                ru[k, j, i] = 1.0 - n / (s * s)
    for k in range(cD):
        for j in range(cH + 1):
            for i in range(cW):
                n = 0
                for sk in range(s):
                    for si in range(s):
                        z, y, x = k * s + sk, j * s, i * s + si
                        n += bool(occ[z, 0, x]) if j == 0 else bool(occ[z, H - 1, x]) if j == cH else \
                            bool(occ[z, y, x] or occ[z, y - 1, x])
                rv[k, j, i] = 1.0 - n / (s * s)
    for k in range(cD + 1):
        for j in range(cH):
            for i in range(cW):
                n = 0
                for sj in range(s):
                    for si in range(s):
                        z, y, x = k * s, j * s + sj, i * s + si
                        n += bool(occ[0, y, x]) if k == 0 else bool(occ[D - 1, y, x]) if k == cD else \
                            bool(occ[z, y, x] or occ[z - 1, y, x])
                rw[k, j, i] = 1.0 - n / (s * s)
    cocc = ((ru[:, :, :-1] == 0) & (ru[:, :, 1:] == 0) & (rv[:, :-1, :] == 0) & (rv[:, 1:, :] == 0) &
            (rw[:-1] == 0) & (rw[1:] == 0))
    cu = np.array([[[sum(u[k * s + sk, j * s + sj, i * s] for sk in range(s) for sj in range(s)) / (s * s)
                     for i in range(cW + 1)] for j in range(cH)] for k in range(cD)])
    cv = np.array([[[sum(v[k * s + sk, j * s, i * s + si] for sk in range(s) for si in range(s)) / (s * s)
                     for i in range(cW)] for j in range(cH + 1)] for k in range(cD)])
    cw = np.array([[[sum(w[k * s, j * s + sj, i * s + si] for sj in range(s) for si in range(s)) / (s * s)
                     for i in range(cW)] for j in range(cH)] for k in range(cD + 1)])
    nb = [((-1, 0, 0), lambda i, j, k: ru[k, j, i]), ((1, 0, 0), lambda i, j, k: ru[k, j, i + 1]),
          ((0, -1, 0), lambda i, j, k: rv[k, j, i]), ((0, 1, 0), lambda i, j, k: rv[k, j + 1, i]),
          ((0, 0, -1), lambda i, j, k: rw[k, j, i]), ((0, 0, 1), lambda i, j, k: rw[k + 1, j, i])]
    inside = lambda i, j, k: 0 <= i < cW and 0 <= j < cH and 0 <= k < cD
    div = np.zeros((cD, cH, cW))
    diag = np.zeros((cD, cH, cW))
    for k in range(cD):
        for j in range(cH):
            for i in range(cW):
                if cocc[k, j, i]:
                    continue
                div[k, j, i] = (cu[k, j, i + 1] - cu[k, j, i]) + (cv[k, j + 1, i] - cv[k, j, i]) + \
                    (cw[k + 1, j, i] - cw[k, j, i])
                d = 0.0
                for (di, dj, dk), r in nb:
                    a, b, c = i + di, j + dj, k + dk
                    if not inside(a, b, c):
                        d += 1.0            # a domain face: weight 1
                    elif not cocc[c, b, a]:
                        d += r(i, j, k)
                diag[k, j, i] = d
    p = np.zeros((cD, cH, cW))
    for _ in range(K):
        for colour in (0, 1):
            for k in range(cD):
                for j in range(cH):
                    for i in range(cW):
                        if (i + j + k) % 2 != colour or cocc[k, j, i] or diag[k, j, i] == 0:
                            continue
                        sm = 0.0
                        for (di, dj, dk), r in nb:
                            a, b, c = i + di, j + dj, k + dk
                            if inside(a, b, c) and not cocc[c, b, a]:
                                sm += r(i, j, k) * p[c, b, a]
                        p[k, j, i] = omega / diag[k, j, i] * (sm - div[k, j, i]) + (1 - omega) * p[k, j, i]
    pp = np.pad(p, 1)   # p = 0 outside the domain
    du = np.where(ru > 0, -(pp[1:-1, 1:-1, 1:] - pp[1:-1, 1:-1, :-1]), 0.0)
    dv = np.where(rv > 0, -(pp[1:-1, 1:, 1:-1] - pp[1:-1, :-1, 1:-1]), 0.0)
    dw = np.where(rw > 0, -(pp[1:, 1:-1, 1:-1] - pp[:-1, 1:-1, 1:-1]), 0.0)
    u, v, w = u.copy(), v.copy(), w.copy()
    free = occ == 0
    for z in range(D):
        for y in range(H):
            for x in range(0, W + 1, s):
                ok = free[z, y, 0] if x == 0 else free[z, y, W - 1] if x == W else free[z, y, x] and free[z, y, x - 1]
                if ok:
                    u[z, y, x] += du[z // s, y // s, x // s]
    for z in range(D):
        for y in range(0, H + 1, s):
            for x in range(W):
                ok = free[z, 0, x] if y == 0 else free[z, H - 1, x] if y == H else free[z, y, x] and free[z, y - 1, x]
                if ok:
                    v[z, y, x] += dv[z // s, y // s, x // s]
    for z in range(0, D + 1, s):
        for y in range(H):
            for x in range(W):
                ok = free[0, y, x] if z == 0 else free[D - 1, y, x] if z == D else free[z, y, x] and free[z - 1, y, x]
                if ok:
                    w[z, y, x] += dw[z // s, y // s, x // s]
    return u, v, w


@pytest.mark.parametrize("s", [2, 4])
def test_coarse_projection_matches_numpy_restatement(oracle64, s):
    """The whole coarse projection with K > 0: the numpy coarse stages, then the
    numpy least-squares block step, against the oracle (FP64; the oracle's
    fused multiply-adds and float block matrix give the tolerance)."""
    W, H, D = 8, 8, 8
    occ = wl.walls_open_top(W, H, D)
    wl.add_box(occ, 3, 4, 2, 5, 3, 3)
    p = wl.smoke_params(W, 7, omega=1.5, solver=capi.SOLVER_COARSE_OPEN)
    p.sub_size = s
    u, v, w = (np.asarray(a, np.float64) for a in wl.initial_velocity(occ, 4, amp=1.0))
    st = {"u": u.copy(), "v": v.copy(), "w": w.copy()}
    assert oracle64.project_coarse(W, H, D, st, occ, p) == 0
    cu, cv, cw = _py_coarse_correction(u, v, w, occ, s, 7, float(np.float32(p.omega)))
    eu, ev, ew = _py_block_projection(cu, cv, cw, occ, s)
    scale = max(np.abs(eu).max(), np.abs(ev).max(), np.abs(ew).max())
    for name, got, exp in (("u", st["u"], eu), ("v", st["v"], ev), ("w", st["w"], ew)):
        np.testing.assert_allclose(got, exp, rtol=0, atol=2e-6 * scale, err_msg=name)
    # the coarse stage did something: without it the result differs
    bu, _, _ = _py_block_projection(u, v, w, occ, s)
    assert np.abs(bu - eu).max() > 1e-3
