"""Seeded synthetic workloads of the smoke step (no dataset is involved).

Inputs are drawn on the host with SplitMix64 so every consumer (the CUDA
library, the CPU oracle, the C++ host API) sees identical bytes:
    x_n = splitmix64(seed + n*0x9E3779B97F4A7C15), u_n = (x_n >> 40) * 2^-24 in [0,1)
and U(a,b) = a + (b-a)*u_n in float32.

Named configurations (cell units, y is up, gravity along -y):
  plain64        64^3, closed walls + open top, sphere source r=6 at (32,8,32),
                 alpha .1 beta .5 eps .2 Tamb 0, attenuation .99, dt .5,
                 omega 1.9, K=200, noise +-1e-3 on live faces (seed 0)
  plain128_obs   128^3, as plain64 plus the box obstacle [48,80]x[56,72]x[48,80]
                 (inclusive), source r=10 at (64,12,64), K=400
  plain256       256^3, walls as plain64, four seeded sphere sources: r~U[8,16],
                 centre x,z~U[r+1, N-r-1], y~U[1, 0.1N], density and temperature
                 ~U[.5,1]; K=600
  plain512       the same at 512^3
  batch64        64 independent instances, edges from {32,48,64,96,128}, each
                 cubic or with one axis doubled; per instance a seeded sphere
                 source (r ~ U[.06,.12] x the shortest edge, in the bottom 15%),
                 alpha ~ U[.05,.2], beta ~ U[.2,.8], eps ~ U[0,.3],
                 dt ~ U[.25,.75]; K=200, 100 steps (batch_mixed())
  control64 / control128  the adjoint problem: plain64's walls, forces
                 (confinement off, dt = 32/N, see control_problem()) and solver at N^3
                 (source r = 6N/64 at (N/2, N/8, N/2)), a zero
                 per-cell control force, 64 steps, and a target density that
                 is a Gaussian blob (sigma 8 cells, peak 1) centred uniformly
                 in the upper half (control_problem())
"Walls closed except an open top" = the open (Dirichlet p=0 outside) solver
with an occupied layer at x=0, x=W-1, y=0, z=0, z=D-1: outside the top face the
pressure is 0, every other side is a solid wall, like ZQ_InitFineGrid3D's
closed layers (ZQ_SmokeSimulationUtils3D.cpp:1535-1584) minus the top one.
Backtrace substeps: 20, the reference default (ZQ_SmokeSimulationUtils3D.cpp:46).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import capi

_GOLD = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, n: int, offset: int = 0) -> np.ndarray:
    idx = np.arange(offset + 1, offset + n + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + idx * _GOLD
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed: int, n: int, offset: int = 0) -> np.ndarray:
    z = splitmix64(seed, n, offset)
    return (z >> np.uint64(40)).astype(np.float32) * np.float32(2.0 ** -24)


def uniform(seed: int, n: int, lo: float, hi: float, offset: int = 0) -> np.ndarray:
    u = uniform01(seed, n, offset)
    lo32, span = np.float32(lo), np.float32(hi) - np.float32(lo)
    return lo32 + span * u


# ---------------------------------------------------------------------------
# occupancy
# ---------------------------------------------------------------------------

def walls_open_top(W: int, H: int, D: int) -> np.ndarray:
    occ = np.zeros((D, H, W), dtype=np.uint8)
    occ[:, :, 0] = 1
    occ[:, :, W - 1] = 1
    occ[:, 0, :] = 1
    occ[0, :, :] = 1
    occ[D - 1, :, :] = 1
    return occ


def walls_closed(W: int, H: int, D: int) -> np.ndarray:
    """ZQ_InitFineGrid3D's six border layers for the closed solvers (Utils3D:1535-1584)."""
    occ = walls_open_top(W, H, D)
    occ[:, H - 1, :] = 1
    return occ


def add_box(occ: np.ndarray, x0: int, x1: int, y0: int, y1: int, z0: int, z1: int) -> np.ndarray:
    """Occupy cells [x0,x1]x[y0,y1]x[z0,z1] (inclusive bounds)."""
    occ[z0:z1 + 1, y0:y1 + 1, x0:x1 + 1] = 1
    return occ


def live_faces(occ: np.ndarray):
    """Open-rule live masks of the u, v, w faces (ZQ_CUDA_Advection3D.cu:471-575)."""
    free = occ == 0
    D, H, W = occ.shape
    lu = np.zeros((D, H, W + 1), bool)
    lu[:, :, 1:W] = free[:, :, 1:] & free[:, :, :-1]
    lu[:, :, 0] = free[:, :, 0]
    lu[:, :, W] = free[:, :, W - 1]
    lv = np.zeros((D, H + 1, W), bool)
    lv[:, 1:H, :] = free[:, 1:, :] & free[:, :-1, :]
    lv[:, 0, :] = free[:, 0, :]
    lv[:, H, :] = free[:, H - 1, :]
    lw = np.zeros((D + 1, H, W), bool)
    lw[1:D] = free[1:] & free[:-1]
    lw[0] = free[0]
    lw[D] = free[D - 1]
    return lu, lv, lw


# ---------------------------------------------------------------------------
# configurations
# ---------------------------------------------------------------------------

@dataclass
class Workload:
    name: str
    W: int
    H: int
    D: int
    params: capi.Params
    occ: np.ndarray
    u: np.ndarray
    v: np.ndarray
    w: np.ndarray
    T: np.ndarray
    rho: np.ndarray
    steps: int
    meta: dict = field(default_factory=dict)

    @property
    def cells(self) -> int:
        return self.W * self.H * self.D

    def state(self) -> dict:
        return {"u": self.u.copy(), "v": self.v.copy(), "w": self.w.copy(), "T": self.T.copy(),
                "rho": self.rho.copy()}


def sphere(cx, cy, cz, r, density=1.0, temperature=1.0) -> capi.Source:
    s = capi.Source()
    s.shape = capi.SOURCE_SPHERE
    s.cx, s.cy, s.cz = cx, cy, cz
    s.hx = s.hy = s.hz = r
    s.density, s.temperature = density, temperature
    return s


def box(cx, cy, cz, hx, hy, hz, density=1.0, temperature=1.0) -> capi.Source:
    s = capi.Source()
    s.shape = capi.SOURCE_BOX
    s.cx, s.cy, s.cz = cx, cy, cz
    s.hx, s.hy, s.hz = hx, hy, hz
    s.density, s.temperature = density, temperature
    return s


def smoke_params(W: int, K: int, *, substeps: int = 20, omega: float = 1.9, vel_mode=capi.ADV_VEL_INMAC_OUTMAC,
                 sca_mode=capi.ADV_SCA_MAC, solver=capi.SOLVER_OPEN) -> capi.Params:
    p = capi.Params()
    p.voxel_size = np.float32(1.0 / W)
    p.step_time = 0.5
    p.substeps = substeps
    p.confine = 0.2
    p.buoyancy = 0.5
    p.gravity = 0.1
    p.tamb = 0.0
    p.vel_atten = p.temp_atten = p.dens_atten = 0.99
    p.solver = solver
    p.sor_iters = K
    p.omega = omega
    p.adv_vel_mode = vel_mode
    p.adv_sca_mode = sca_mode
    p.backtrace_full = 0
    p.n_sources = 0
    return p


def initial_velocity(occ: np.ndarray, seed: int, amp: float = 1e-3):
    D, H, W = occ.shape
    lu, lv, lw = live_faces(occ)
    nu, nv, nw = lu.size, lv.size, lw.size
    u = uniform(seed, nu, -amp, amp, 0).reshape(lu.shape)
    v = uniform(seed, nv, -amp, amp, nu).reshape(lv.shape)
    w = uniform(seed, nw, -amp, amp, nu + nv).reshape(lw.shape)
    u[~lu] = 0
    v[~lv] = 0
    w[~lw] = 0
    return u, v, w


def plain_sources(N: int, seed: int) -> list:
    """Four seeded sphere sources near the floor of an N^3 domain."""
    rs = uniform(seed + 1000, 4, 8.0, 16.0)
    src = []
    for q in range(4):
        r = float(rs[q])
        u3 = uniform01(seed + 2000 + q, 5)
        cx = float(np.float32(r + 1) + np.float32(N - 2 * r - 2) * u3[0])
        cz = float(np.float32(r + 1) + np.float32(N - 2 * r - 2) * u3[1])
        cy = float(np.float32(1.0) + np.float32(0.1 * N - 1.0) * u3[2])
        den = float(np.float32(0.5) + np.float32(0.5) * u3[3])
        tem = float(np.float32(0.5) + np.float32(0.5) * u3[4])
        src.append(sphere(cx, cy, cz, r, den, tem))
    return src


def make(name: str, *, K: int | None = None, substeps: int = 20, steps: int | None = None, seed: int = 0,
         vel_mode=capi.ADV_VEL_INMAC_OUTMAC, sca_mode=capi.ADV_SCA_MAC, omega: float = 1.9) -> Workload:
    if name in ("plain64", "plain128_obs"):
        N = 64 if name == "plain64" else 128
        occ = walls_open_top(N, N, N)
        if name == "plain64":
            src = [sphere(32.0, 8.0, 32.0, 6.0)]
            Kd, steps_d = 200, 100
        else:
            add_box(occ, 48, 80, 56, 72, 48, 80)
            src = [sphere(64.0, 12.0, 64.0, 10.0)]
            Kd, steps_d = 400, 500
    elif name.startswith("plain") and name[5:].isdigit():
        N = int(name[5:])
        occ = walls_open_top(N, N, N)
        src = plain_sources(N, seed)
        Kd, steps_d = 600, 200
    elif name.startswith("coarse") and name[6:].isdigit():
        # the reference's fine256 configuration (expsimu3D/fine256.txt): open
        # domain, the centred sphere obstacle of intObj sphere (Utils3D:1587-1599,
        # r^2 < N^2/400), COARSE_OPEN_POISSON_SOR with subSize 8, maxIter 600,
        # regular-grid advection (inReg_outReg, Reg); sources as plainN
        N = int(name[6:])
        occ = np.zeros((N, N, N), np.uint8)
        c = np.arange(N) + 0.5 - N / 2
        occ[(c[:, None, None] ** 2 + c[None, :, None] ** 2 + c[None, None, :] ** 2) < N * N / 400.0] = 1
        src = plain_sources(N, seed)
        Kd, steps_d = 600, 200
        vel_mode, sca_mode = capi.ADV_VEL_INREG_OUTREG, capi.ADV_SCA_REG
    else:
        raise KeyError(f"unknown workload {name!r}")
    N = occ.shape[0]
    p = smoke_params(N, K if K is not None else Kd, substeps=substeps, omega=omega, vel_mode=vel_mode,
                     sca_mode=sca_mode)
    if name.startswith("coarse"):
        p.solver = capi.SOLVER_COARSE_OPEN
        p.sub_size = 8
    p.set_sources(src)
    u, v, w = initial_velocity(occ, seed)
    T = np.zeros((N, N, N), np.float32)
    rho = np.zeros((N, N, N), np.float32)
    return Workload(name, N, N, N, p, occ, u, v, w, T, rho, steps if steps is not None else steps_d,
                    {"seed": seed, "K": p.sor_iters, "substeps": substeps})


def small_case(W: int, H: int, D: int, *, seed: int = 7, K: int = 20, substeps: int = 4, obstacle: bool = True,
               closed: bool = False, vel_amp: float = 0.05, scalars: bool = True,
               vel_mode=capi.ADV_VEL_INMAC_OUTMAC, sca_mode=capi.ADV_SCA_MAC, omega: float = 1.9) -> Workload:
    """A small, irregular, fully seeded case for parity tests (odd sizes allowed)."""
    occ = walls_closed(W, H, D) if closed else walls_open_top(W, H, D)
    if obstacle and min(W, H, D) >= 6:
        add_box(occ, W // 3, W // 3 + 1, H // 2, H // 2 + 1, D // 3, D // 2)
    p = smoke_params(W, K, substeps=substeps, omega=omega, vel_mode=vel_mode, sca_mode=sca_mode,
                     solver=capi.SOLVER_CLOSED if closed else capi.SOLVER_OPEN)
    p.step_time = 0.05
    p.set_sources([sphere(W / 2, min(2.5, H / 3), D / 2, max(1.5, W / 6)),
                   box(W / 4, H / 4 + 0.5, D / 2, 1.0, 1.0, 1.5, 0.7, 0.4)])
    u, v, w = initial_velocity(occ, seed, amp=vel_amp)
    if scalars:
        T = uniform(seed + 1, W * H * D, 0.0, 1.0).reshape(D, H, W)
        rho = uniform(seed + 2, W * H * D, 0.0, 1.0).reshape(D, H, W)
    else:
        T = np.zeros((D, H, W), np.float32)
        rho = np.zeros((D, H, W), np.float32)
    return Workload(f"small{W}x{H}x{D}", W, H, D, p, occ, u, v, w, T, rho, 1, {"seed": seed})


def batch_member(idx: int, *, seed: int = 0, K: int = 200, edges=(32, 48, 64, 96, 128)) -> Workload:
    """Instance idx of the mixed-size batch (all draws seeded by seed and idx)."""
    base = seed * 1_000_003 + 7919 * (idx + 1)
    u = uniform01(base, 16)
    e = int(edges[min(len(edges) - 1, int(u[0] * len(edges)))])
    dims = [e, e, e]
    if u[1] >= 0.5:                        # one axis doubled
        dims[min(2, int(u[2] * 3))] *= 2
    W, H, D = dims
    occ = walls_open_top(W, H, D)
    m = min(W, H, D)
    r = float(np.float32(m) * (np.float32(0.06) + np.float32(0.06) * u[3]))
    cx = float(np.float32(r + 1) + np.float32(W - 2 * r - 2) * u[4])
    cz = float(np.float32(r + 1) + np.float32(D - 2 * r - 2) * u[5])
    cy = float(np.float32(1.0) + np.float32(max(0.15 * H - 1.0, 0.0)) * u[6])
    p = smoke_params(W, K)
    p.gravity = float(np.float32(0.05) + np.float32(0.15) * u[7])      # alpha (density)
    p.buoyancy = float(np.float32(0.2) + np.float32(0.6) * u[8])       # beta (temperature)
    p.confine = float(np.float32(0.3) * u[9])                          # eps
    p.step_time = float(np.float32(0.25) + np.float32(0.5) * u[10])    # dt
    p.set_sources([sphere(cx, cy, cz, r)])
    uu, vv, ww = initial_velocity(occ, base + 17)
    T = np.zeros((D, H, W), np.float32)
    rho = np.zeros((D, H, W), np.float32)
    return Workload(f"batch[{idx}]{W}x{H}x{D}", W, H, D, p, occ, uu, vv, ww, T, rho, 100,
                    {"seed": seed, "index": idx, "K": K})


def batch_mixed(n: int = 64, *, seed: int = 0, K: int = 200, edges=(32, 48, 64, 96, 128)) -> list[Workload]:
    """The mixed-size batch: n seeded instances (batch_member(0..n-1))."""
    return [batch_member(i, seed=seed, K=K, edges=edges) for i in range(n)]


def control_problem(N: int = 64, *, seed: int = 0, K: int = 200, nsteps: int = 64, substeps: int = 20,
                    sigma: float = 8.0, confine: float = 0.0, dt: float | None = None):
    """The force-field control problem at N^3: (workload, target density).

    Loss L(F) = sum_cells (rho_final - target)^2 after nsteps steps with the
    per-cell force F (3, N, N, N) added every step; F = 0 initially.

    Vorticity confinement is off by default: its normal N = grad|w| / |grad|w||
    (ZQ_CUDA_AddForce3D.cu:64-111) has a derivative that grows as
    1/|grad|w|| where the vorticity is nearly uniform, and over tens of steps
    the exact gradient of the rollout grows without bound (measured at 64^3:
    |dL/dF| ~ 1e3 for 16 steps, ~ 1e6 at 32, ~ 1e16 at 64 with eps = 0.2, where
    FP32 and FP64 gradients and finite differences no longer agree).

    dt defaults to 32/N (0.5 at 64^3, 0.25 at 128^3): the same distance in
    cells per step at every resolution.  The backtrace chains 19 substeps;
    at 128^3 with dt = 0.5 the plume moves ~2.3 cells per substep and the
    exact gradient is ill-conditioned (|dL/dF| ~ 1e5 after 8 steps, 1e15
    after 64, FP32 and FP64 gradients 1.5e-2 apart after 8 steps); with
    dt = 0.25 it stays ~1e3 over 64 steps."""
    occ = walls_open_top(N, N, N)
    p = smoke_params(N, K, substeps=substeps)
    p.confine = confine
    p.step_time = float(np.float32(32.0 / N)) if dt is None else dt
    p.set_sources([sphere(N / 2, N / 8, N / 2, 6.0 * N / 64)])
    u, v, w = initial_velocity(occ, seed)
    T = np.zeros((N, N, N), np.float32)
    rho = np.zeros((N, N, N), np.float32)
    wl = Workload(f"control{N}", N, N, N, p, occ, u, v, w, T, rho, nsteps, {"seed": seed, "K": K})
    c = uniform01(seed + 4242, 3)
    cx = float(np.float32(sigma) + np.float32(N - 2 * sigma) * c[0])
    cy = float(np.float32(N / 2) + np.float32(N / 2 - sigma) * c[1])
    cz = float(np.float32(sigma) + np.float32(N - 2 * sigma) * c[2])
    z, y, x = np.meshgrid(np.arange(N) + 0.5, np.arange(N) + 0.5, np.arange(N) + 0.5, indexing="ij")
    r2 = (x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2
    target = np.exp(-r2 / (2.0 * sigma * sigma)).astype(np.float32)
    wl.meta.update({"target_centre": (cx, cy, cz), "sigma": sigma})
    return wl, target
