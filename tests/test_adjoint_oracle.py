"""CPU: the oracle's reverse mode (FP64) against transposition identities and
central finite differences of its own FP64 forward.

These pin the FP64 CPU gradient that the GPU adjoint is compared with:
  * linear stages (projection, scalar advection at fixed velocity) satisfy
    <A x, y> = <x, A^T y> to rounding;
  * nonlinear stages (velocity advection, forces) and the whole control
    problem match central differences (h = 1e-6 in FP64) to 1e-6 relative.
"""
import numpy as np
import pytest

from zq_smokesimulation_gb300 import capi
from zq_smokesimulation_gb300 import workloads as wl

FD_TOL = 1e-6


def generic_velocity(st, rng, amp=0.3):
    """Random velocity on every face: with exactly zero velocity in a pocket,
    backtrace points sit on lattice planes where trilinear interpolation has a
    kink and central differences average the one-sided derivatives."""
    for k in "uvw":
        st[k] = rng.standard_normal(st[k].shape) * amp
    return st


def dot(a, b):
    return float(np.sum(np.asarray(a, np.float64) * np.asarray(b, np.float64)))


def central(f, h=1e-6):
    return (f(h) - f(-h)) / (2 * h)


@pytest.mark.parametrize("closed", [False, True])
def test_project_adjoint_is_transpose(oracle64, closed):
    rng = np.random.default_rng(1)
    w = wl.small_case(11, 9, 7, K=6, closed=closed)
    W, H, D = w.W, w.H, w.D
    x = {k: rng.standard_normal(getattr(w, k).shape) for k in "uvw"}
    y = {k: rng.standard_normal(getattr(w, k).shape) for k in "uvw"}
    px = {k: x[k].copy() for k in "uvw"}
    oracle64.project(W, H, D, px, w.occ, w.params)
    pty = {k: y[k].copy() for k in "uvw"}
    oracle64.project_adjoint(W, H, D, pty, w.occ, w.params)
    a = sum(dot(px[k], y[k]) for k in "uvw")
    b = sum(dot(x[k], pty[k]) for k in "uvw")
    assert abs(a - b) <= 1e-12 * abs(a)


def test_advect_scalar_adjoint(oracle64):
    rng = np.random.default_rng(2)
    w = wl.small_case(10, 9, 7, K=4, vel_amp=0.4, substeps=4)
    w.params.step_time = 0.3
    W, H, D = w.W, w.H, w.D
    st = generic_velocity(oracle64.state(w), rng)
    T, R = rng.standard_normal((D, H, W)), rng.standard_normal((D, H, W))
    gT, gR = rng.standard_normal((D, H, W)), rng.standard_normal((D, H, W))
    gTin, gRin, gv = oracle64.advect_scalar_adjoint(W, H, D, st, w.occ, T, R, gT, gR, w.params)

    def out(vel):
        s = {k: vel[k] for k in "uvw"}
        s["T"], s["rho"] = T.copy(), R.copy()
        oracle64.advect_scalar(W, H, D, s, w.occ, w.params, capi.ADV_SCA_MAC)
        return s

    s = out(st)
    assert abs((dot(s["T"], gT) + dot(s["rho"], gR)) - (dot(T, gTin) + dot(R, gRin))) <= 1e-12 * abs(dot(T, gTin))
    dv = {k: rng.standard_normal(st[k].shape) for k in "uvw"}

    def L(h):
        s = out({k: st[k] + h * dv[k] for k in "uvw"})
        return dot(s["T"], gT) + dot(s["rho"], gR)

    fd, an = central(L), sum(dot(gv[k], dv[k]) for k in "uvw")
    assert abs(fd - an) <= FD_TOL * abs(an)


def test_advect_velocity_adjoint(oracle64):
    rng = np.random.default_rng(3)
    w = wl.small_case(10, 9, 7, K=4, vel_amp=0.4, substeps=5)
    w.params.step_time = 0.3
    W, H, D = w.W, w.H, w.D
    st = generic_velocity(oracle64.state(w), rng)
    g3 = {k: rng.standard_normal(st[k].shape) for k in "uvw"}
    g2 = oracle64.advect_velocity_adjoint(W, H, D, st, w.occ, w.params, g3)
    dv = {k: rng.standard_normal(st[k].shape) for k in "uvw"}

    def L(h):
        s = {k: st[k] + h * dv[k] for k in "uvw"}
        s["T"], s["rho"] = st["T"], st["rho"]
        oracle64.advect_velocity(W, H, D, s, w.occ, w.params, capi.ADV_VEL_INMAC_OUTMAC, True)
        return sum(dot(s[k], g3[k]) for k in "uvw")

    fd, an = central(L), sum(dot(g2[k], dv[k]) for k in "uvw")
    assert abs(fd - an) <= FD_TOL * abs(an)


def test_add_force_adjoint(oracle64):
    rng = np.random.default_rng(4)
    w = wl.small_case(10, 9, 8, K=4, vel_amp=0.4)
    w.params.confine = 1.5
    W, H, D = w.W, w.H, w.D
    st = generic_velocity(oracle64.state(w), rng)
    F0 = rng.standard_normal((3, D, H, W)) * 0.1
    gvel = {k: rng.standard_normal(st[k].shape) for k in "uvw"}
    dvel = {k: rng.standard_normal(st[k].shape) for k in "uvw"}
    dT, dR, dF = (rng.standard_normal((D, H, W)), rng.standard_normal((D, H, W)),
                  rng.standard_normal((3, D, H, W)))
    g = {k: gvel[k].copy() for k in "uvw"}
    gT, gR, gF = np.zeros((D, H, W)), np.zeros((D, H, W)), np.zeros((3, D, H, W))
    oracle64.add_force_adjoint(W, H, D, st, w.occ, w.params, g, gT, gR, gF)

    def L(h):
        s = {k: st[k] + h * dvel[k] for k in "uvw"}
        s["T"], s["rho"] = st["T"] + h * dT, st["rho"] + h * dR
        oracle64.add_force_ctrl(W, H, D, s, w.occ, w.params, F0 + h * dF)
        return sum(dot(s[k], gvel[k]) for k in "uvw")

    fd = central(L)
    an = sum(dot(g[k], dvel[k]) for k in "uvw") + dot(gT, dT) + dot(gR, dR) + dot(gF, dF)
    assert abs(fd - an) <= FD_TOL * abs(an)


@pytest.mark.parametrize("closed", [False, True])
def test_control_gradient_matches_fd(oracle64, closed):
    """dL/dF of the full multi-step problem along seeded directions."""
    rng = np.random.default_rng(5)
    w = wl.small_case(10, 9, 8, K=6, vel_amp=0.2, substeps=3, closed=closed)
    w.params.step_time, w.params.confine = 0.2, 0.5
    W, H, D = w.W, w.H, w.D
    st = oracle64.state(w)
    target = rng.random((D, H, W))
    F = rng.standard_normal((3, D, H, W)) * 0.05
    nsteps = 3
    L0, gF, g0 = oracle64.control_loss(W, H, D, st, w.occ, w.params, nsteps, F, target, grad=True)
    assert np.isfinite(L0) and np.abs(gF).max() > 0
    for _ in range(3):
        d = rng.standard_normal((3, D, H, W))
        fd = central(lambda h: oracle64.control_loss(W, H, D, st, w.occ, w.params, nsteps, F + h * d, target))
        an = dot(gF, d)
        assert abs(fd - an) <= FD_TOL * abs(an), (fd, an)


def test_step_adjoint_rejects_regular_modes(oracle64):
    w = wl.small_case(8, 8, 8, K=2, vel_mode=capi.ADV_VEL_INREG_OUTREG)
    st = oracle64.state(w)
    g = {k: np.zeros_like(v) for k, v in st.items()}
    gF = np.zeros((3, 8, 8, 8))
    assert oracle64.step_adjoint(8, 8, 8, st, w.occ, w.params, None, g, gF) == capi.ZQS_EUNSUPPORTED
