"""GPU: the external control force and the reverse mode (zqs_adjoint_*).

* The forward with a control force is bit-identical to the FP32 oracle.
* The GPU gradient dL/dF (FP32, atomics) matches the FP64 CPU gradient of the
  oracle's reverse mode within 1e-3 relative (observed ~1e-6), and central
  finite differences of the FP64 oracle forward along seeded unit directions.
* The checkpoint spacing does not change the gradient (beyond the last-bit
  variation of atomic accumulation).
"""
import numpy as np
import pytest

from conftest import rel_l2
from zq_smokesimulation_gb300 import capi
from zq_smokesimulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

FIELDS = ("u", "v", "w", "T", "rho")
GRAD_TOL = 1e-3


def make_grid(w):
    g = capi.Grid(w.W, w.H, w.D)
    g.set_params(w.params)
    g.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
    return g


def control_case(dims=(16, 14, 12), K=10, substeps=3, closed=False, seed=11):
    rng = np.random.default_rng(seed)
    w = wl.small_case(*dims, K=K, vel_amp=0.2, substeps=substeps, closed=closed)
    w.params.step_time, w.params.confine = 0.2, 0.5
    target = rng.random((w.D, w.H, w.W)).astype(np.float32)
    F = (rng.standard_normal((3, w.D, w.H, w.W)) * 0.05).astype(np.float32)
    return w, F, target


def gpu_gradient(w, F, target, nsteps, every):
    g = make_grid(w)
    a = capi.Adjoint(g, nsteps, every)
    a.forward(F)
    rho = g.download(capi.FIELD_DENSITY)
    gF = a.backward(2.0 * (rho - target))
    return rho, gF, a, g


def test_force_forward_bitwise(zqs_lib, oracle32):
    w, F, _ = control_case((17, 13, 11), K=8)
    F = F * 6
    g = make_grid(w)
    g.set_force(F)
    g.step(3)
    st = oracle32.state(w)
    assert oracle32.step_ctrl(w.W, w.H, w.D, st, w.occ, w.params, F, 3) == 0
    out = g.state()
    for k in FIELDS:
        assert np.array_equal(out[k], st[k]), k
    # removing the force gives the plain step again
    g2 = make_grid(w)
    g2.set_force(F)
    g2.set_force(None)
    g2.step(2)
    st = oracle32.state(w)
    oracle32.step(w.W, w.H, w.D, st, w.occ, w.params, 2)
    out = g2.state()
    for k in FIELDS:
        assert np.array_equal(out[k], st[k]), k


@pytest.mark.parametrize("closed", [False, True])
def test_gradient_matches_fp64_cpu(zqs_lib, oracle64, closed):
    w, F, target = control_case(closed=closed)
    nsteps = 4
    rho, gF, a, g = gpu_gradient(w, F, target, nsteps, 2)
    L64, gF64, g0 = oracle64.control_loss(w.W, w.H, w.D, oracle64.state(w), w.occ, w.params, nsteps, F, target,
                                          grad=True)
    e = rel_l2(gF, gF64)
    assert e <= GRAD_TOL, e
    # adjoint of the initial density (last block of the packed initial-state adjoint)
    n = w.W * w.H * w.D
    g_rho0 = a.initial_adjoint(capi.FIELD_DENSITY)
    assert rel_l2(g_rho0, g0[-n:].reshape(w.D, w.H, w.W)) <= GRAD_TOL
    nu = (w.W + 1) * w.H * w.D
    g_u0 = a.initial_adjoint(capi.FIELD_U)
    assert rel_l2(g_u0, g0[:nu].reshape(w.D, w.H, w.W + 1)) <= GRAD_TOL
    inf = a.info()
    assert inf.checkpoints == 3 and inf.launches_backward > 0 and inf.device_bytes > 0


def test_gradient_matches_central_differences(zqs_lib, oracle64):
    """Directional derivatives along seeded unit directions d.  The loss is
    only piecewise smooth (trilinear interpolation), so central differences
    carry an O(h^2)-plus-kink error: with h = 1e-5 they match to 1e-3
    relative; with h = 1e-3 the error is measured against |g| |d|."""
    w, F, target = control_case(K=12, substeps=4)
    nsteps = 5
    _, gF, _, _ = gpu_gradient(w, F, target, nsteps, 2)
    gnorm = float(np.linalg.norm(gF.astype(np.float64)))
    rng = np.random.default_rng(7)
    st = oracle64.state(w)

    def fd(d, h):
        lp = oracle64.control_loss(w.W, w.H, w.D, st, w.occ, w.params, nsteps, F + h * d, target)
        lm = oracle64.control_loss(w.W, w.H, w.D, st, w.occ, w.params, nsteps, F - h * d, target)
        return (lp - lm) / (2 * h)

    for _ in range(4):
        d = rng.standard_normal(F.shape)
        d /= np.linalg.norm(d)
        an = float(np.sum(gF.astype(np.float64) * d))
        f5 = fd(d, 1e-5)
        assert abs(f5 - an) <= GRAD_TOL * abs(f5), (f5, an)
        f3 = fd(d, 1e-3)
        assert abs(f3 - an) <= GRAD_TOL * gnorm, (f3, an, gnorm)


def test_checkpoint_spacing_invariant(zqs_lib):
    w, F, target = control_case()
    nsteps = 5
    grads = [gpu_gradient(w, F, target, nsteps, every)[1] for every in (1, 2, 3, 5)]
    for gF in grads[1:]:
        assert rel_l2(gF, grads[0]) <= 1e-5


def test_default_substeps_and_zero_control(zqs_lib, oracle64):
    """20 backtrace substeps (the reference default) and F = 0, as in the
    control problem; small grid."""
    w, _, target = control_case((14, 12, 10), K=8, substeps=20)
    F = np.zeros((3, w.D, w.H, w.W), np.float32)
    nsteps = 3
    _, gF, _, _ = gpu_gradient(w, F, target, nsteps, 3)
    _, gF64, _ = oracle64.control_loss(w.W, w.H, w.D, oracle64.state(w), w.occ, w.params, nsteps, F, target,
                                       grad=True)
    assert rel_l2(gF, gF64) <= GRAD_TOL


def test_adjoint_rejects_unsupported(zqs_lib):
    w = wl.small_case(8, 8, 8, K=2, vel_mode=capi.ADV_VEL_INREG_OUTREG)
    g = make_grid(w)
    with pytest.raises(capi.ZQSError) as e:
        capi.Adjoint(g, 2)
    assert e.value.code == capi.ZQS_EUNSUPPORTED
    w = wl.small_case(8, 8, 8, K=2, substeps=40)
    g = make_grid(w)
    with pytest.raises(capi.ZQSError) as e:
        capi.Adjoint(g, 2)
    assert e.value.code == capi.ZQS_EUNSUPPORTED
    w = wl.small_case(8, 8, 8, K=2)
    g = make_grid(w)
    a = capi.Adjoint(g, 2)
    with pytest.raises(capi.ZQSError) as e:
        a.backward(np.zeros((8, 8, 8), np.float32))
    assert e.value.code == capi.ZQS_ENOTREADY


def test_torch_autograd_function(zqs_lib, oracle64):
    torch = pytest.importorskip("torch")
    from zq_smokesimulation_gb300.torch_ops import SmokeControl
    w, F, target = control_case()
    nsteps = 3
    g = make_grid(w)
    ctl = SmokeControl(g, w.state(), nsteps, checkpoint_every=2)
    Ft = torch.tensor(F, device="cuda", requires_grad=True)
    tt = torch.tensor(target, device="cuda")
    rho = ctl(Ft)
    loss = ((rho - tt) ** 2).sum()
    loss.backward()
    L64, gF64, _ = oracle64.control_loss(w.W, w.H, w.D, oracle64.state(w), w.occ, w.params, nsteps, F, target,
                                         grad=True)
    assert abs(float(loss.detach()) - L64) <= 1e-4 * abs(L64)
    assert rel_l2(Ft.grad.cpu().numpy(), gF64) <= GRAD_TOL
    # a second evaluation restarts from the initial state
    rho2 = ctl(Ft.detach())
    assert torch.equal(rho2, rho.detach())


def _control64_check(ndirs, seed=0):
    """The control problem at 64^3 (64 steps, checkpoints every 8): GPU
    gradient against the FP64 CPU gradient, and against FP64 central
    differences along ndirs seeded unit directions (h = 1e-3)."""
    import json
    import os

    from oracle.binding import Oracle
    o64 = Oracle(np.float64)
    w, target = wl.control_problem(64, seed=seed)
    F = np.zeros((3, 64, 64, 64), np.float32)
    rho, gF, a, g = gpu_gradient(w, F, target, w.steps, 8)
    L64, gF64, _ = o64.control_loss(64, 64, 64, o64.state(w), w.occ, w.params, w.steps, F, target, grad=True)
    gnorm = float(np.linalg.norm(gF64))
    rel64 = rel_l2(gF, gF64)
    rng = np.random.default_rng(1234 + seed)
    st = o64.state(w)
    errs = []
    for _ in range(ndirs):
        d = rng.standard_normal(F.shape)
        d /= np.linalg.norm(d)
        h = 1e-3
        lp = o64.control_loss(64, 64, 64, st, w.occ, w.params, w.steps, F + h * d, target)
        lm = o64.control_loss(64, 64, 64, st, w.occ, w.params, w.steps, F - h * d, target)
        fd = (lp - lm) / (2 * h)
        an = float(np.sum(gF.astype(np.float64) * d))
        errs.append({"fd": fd, "gpu": an, "err_rel_fd": abs(fd - an) / abs(fd),
                     "err_rel_gnorm": abs(fd - an) / gnorm})
    report = {"problem": "control64", "steps": w.steps, "loss_fp64": L64, "grad_norm_fp64": gnorm,
              "rel_l2_gpu_vs_fp64": rel64, "directions": ndirs,
              "max_err_rel_gnorm": max(e["err_rel_gnorm"] for e in errs),
              "median_err_rel_fd": float(np.median([e["err_rel_fd"] for e in errs]))}
    print(json.dumps(report))
    out = os.environ.get("ZQS_ADJOINT_REPORT")
    if out:
        with open(out, "w") as fh:
            json.dump({"summary": report, "directions": errs}, fh, indent=1)
    return rel64, errs, gnorm


@pytest.mark.slow
def test_control64_gradient(zqs_lib):
    """Configuration 4 at 64^3 (64 steps, checkpoints every 8; confinement off
    and dt = 32/N, workloads.control_problem): GPU gradient within 1e-3 of the
    FP64 CPU gradient, and FP64 central differences (h = 1e-3) along 8 seeded
    unit directions within 1e-3 of |grad L|."""
    rel64, errs, gnorm = _control64_check(8)
    assert rel64 <= GRAD_TOL
    for e in errs:
        assert e["err_rel_gnorm"] <= GRAD_TOL, e


@pytest.mark.long
def test_control64_gradient_32_directions(zqs_lib):
    """The same with the 32 directions of the configuration (--runlong)."""
    rel64, errs, gnorm = _control64_check(32)
    assert rel64 <= GRAD_TOL
    for e in errs:
        assert e["err_rel_gnorm"] <= GRAD_TOL, e
