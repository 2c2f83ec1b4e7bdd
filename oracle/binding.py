"""ctypes binding of the CPU oracle (oracle/_build/libzqs_oracle.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline / reference arm of bench.py, always to check results.  The oracle
restates the reference's per-timestep path (see zqs_oracle.cpp); the GPU tests
pin it to the reference's own kernels for every stage but the SOR, whose
source is not in the reference tree (tests/test_ref_pin_gpu.py).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_libs: dict = {}


def load():
    if "lib" in _libs:
        return _libs["lib"]
    from . import build as _b  # type: ignore
    path = _b.build()
    lib = C.CDLL(str(path))
    _libs["lib"] = lib
    return lib


def _p(a):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return C.c_void_p(a.ctypes.data)


class Oracle:
    """Oracle in FP32 (dtype=np.float32) or FP64 (np.float64)."""

    def __init__(self, dtype=np.float32):
        self.lib = load()
        self.dtype = np.dtype(dtype)
        self.sfx = "f32" if self.dtype == np.float32 else "f64"

    def _f(self, name):
        return getattr(self.lib, f"zqo_{name}_{self.sfx}")

    def arr(self, a):
        return np.ascontiguousarray(a, dtype=self.dtype)

    def mac_to_regular4(self, W, H, D, u, v, w):
        out = np.empty((D, H, W, 4), self.dtype)
        self._f("mac_to_regular4")(W, H, D, _p(u), _p(v), _p(w), _p(out))
        return out

    def regular4_to_mac(self, W, H, D, vel4):
        u = np.empty((D, H, W + 1), self.dtype)
        v = np.empty((D, H + 1, W), self.dtype)
        w = np.empty((D + 1, H, W), self.dtype)
        v4 = self.arr(vel4)  # held: a converted temporary must outlive the call
        self._f("regular4_to_mac")(W, H, D, _p(v4), _p(u), _p(v), _p(w))
        return u, v, w

    def vorticity(self, W, H, D, u, v, w, h):
        vort = np.empty((D, H, W, 3), self.dtype)
        vs = np.empty((D, H, W), self.dtype)
        u, v, w = self.arr(u), self.arr(v), self.arr(w)
        self._f("vorticity")(W, H, D, _p(u), _p(v), _p(w),
                             (C.c_float if self.sfx == "f32" else C.c_double)(h), _p(vort), _p(vs))
        return vort, vs

    def add_force(self, W, H, D, st, occ, params):
        self._f("add_force")(W, H, D, _p(st["u"]), _p(st["v"]), _p(st["w"]), _p(occ), _p(st["T"]), _p(st["rho"]),
                             C.byref(params))

    def attenuate(self, W, H, D, st, occ, params):
        self._f("attenuate")(W, H, D, _p(st["u"]), _p(st["v"]), _p(st["w"]), _p(st["T"]), _p(st["rho"]), _p(occ),
                             C.byref(params))

    def advect_velocity(self, W, H, D, st, occ, params, mode, is_open=True):
        return self._f("advect_velocity")(W, H, D, _p(st["u"]), _p(st["v"]), _p(st["w"]), _p(occ),
                                          C.byref(params), mode, 1 if is_open else 0)

    def advect_scalar(self, W, H, D, st, occ, params, mode):
        return self._f("advect_scalar")(W, H, D, _p(st["u"]), _p(st["v"]), _p(st["w"]), _p(occ), _p(st["T"]),
                                        _p(st["rho"]), _p(st["T"]), _p(st["rho"]), C.byref(params), mode)

    def project(self, W, H, D, st, occ, params, want=False):
        from zq_smokesimulation_gb300 import capi
        p = np.zeros((D, H, W), self.dtype)
        div = np.zeros((D, H, W), self.dtype)
        stats = capi.Stats()
        self._f("project")(W, H, D, _p(st["u"]), _p(st["v"]), _p(st["w"]), _p(occ), C.byref(params), _p(p), _p(div),
                           C.byref(stats))
        return (p, div, stats) if want else stats

    def project_coarse(self, W, H, D, st, occ, params):
        """Coarse-grid projection in place on st's u, v, w (ZQS_SOLVER_COARSE_OPEN)."""
        return self._f("project_coarse")(W, H, D, _p(st["u"]), _p(st["v"]), _p(st["w"]), _p(occ),
                                         C.byref(params))

    def stamp_objects(self, W, H, D, st, occ, objs, closed, params):
        """In place on occ (uint8, (D, H, W)) and st's u, v, w."""
        from zq_smokesimulation_gb300 import capi
        arr, keep = capi.make_objects(objs)
        assert occ.dtype == np.uint8 and occ.flags["C_CONTIGUOUS"]
        self._f("stamp_objects")(W, H, D, _p(occ), _p(st["u"]), _p(st["v"]), _p(st["w"]),
                                 C.cast(arr, C.c_void_p), len(objs), int(closed), C.byref(params))
        del keep

    def render(self, vol, cam):
        """Ray march a dense (D, H, W) density; returns (height, width, 4), bottom row first."""
        v = self.arr(vol)
        out = np.zeros((cam.height, cam.width, 4), self.dtype)
        self._f("render")(_p(v), v.shape[2], v.shape[1], v.shape[0], C.byref(cam), _p(out))
        return out

    def submatrix(self, s):
        """The sub-projection matrix of block edge s as (3 s^2 (s-1), 3 s^2 (s+1)) float32."""
        rows, cols = 3 * s * s * (s - 1), 3 * s * s * (s + 1)
        out = np.zeros((rows, cols), np.float32)
        n = self.lib.zqo_submatrix(s, _p(out), rows * cols)
        assert n == rows * cols, n
        return out

    def reinject(self, W, H, D, st, params):
        self._f("reinject")(W, H, D, _p(st["T"]), _p(st["rho"]), C.byref(params))

    def step(self, W, H, D, st, occ, params, nsteps=1):
        p = np.zeros((D, H, W), self.dtype)
        rc = self._f("step")(W, H, D, _p(st["u"]), _p(st["v"]), _p(st["w"]), _p(st["T"]), _p(st["rho"]), _p(occ),
                             C.byref(params), nsteps, _p(p))
        return rc, p

    # -- control problem and reverse mode ------------------------------------------
    def step_ctrl(self, W, H, D, st, occ, params, F, nsteps=1):
        """nsteps steps with the external per-cell force F (3, D, H, W)."""
        Fa = self.arr(F)
        return self._f("step_ctrl")(W, H, D, _p(st["u"]), _p(st["v"]), _p(st["w"]), _p(st["T"]), _p(st["rho"]),
                                    _p(occ), C.byref(params), nsteps, _p(Fa))

    def add_force_ctrl(self, W, H, D, st, occ, params, F):
        Fa = self.arr(F)
        self._f("add_force_ctrl")(W, H, D, _p(st["u"]), _p(st["v"]), _p(st["w"]), _p(occ), _p(st["T"]),
                                  _p(st["rho"]), C.byref(params), _p(Fa))

    def project_adjoint(self, W, H, D, g, occ, params):
        """In place on g = {u, v, w}: adjoint of the projected velocity -> of the input."""
        self._f("project_adjoint")(W, H, D, _p(g["u"]), _p(g["v"]), _p(g["w"]), _p(occ), C.byref(params))

    def advect_scalar_adjoint(self, W, H, D, vel, occ, Tin, Din, gT, gD, params):
        """Returns (gTin, gDin, gvel) for the MAC-velocity scalar advection."""
        gTin = np.zeros((D, H, W), self.dtype)
        gDin = np.zeros((D, H, W), self.dtype)
        gv = {k: np.zeros_like(self.arr(vel[k])) for k in ("u", "v", "w")}
        Tin, Din, gT, gD = self.arr(Tin), self.arr(Din), self.arr(gT), self.arr(gD)
        self._f("advect_scalar_adjoint")(W, H, D, _p(vel["u"]), _p(vel["v"]), _p(vel["w"]), _p(occ),
                                         _p(Tin), _p(Din), _p(gT), _p(gD),
                                         _p(gTin), _p(gDin), _p(gv["u"]), _p(gv["v"]), _p(gv["w"]), C.byref(params))
        return gTin, gDin, gv

    def advect_velocity_adjoint(self, W, H, D, vel, occ, params, g3):
        g2 = {k: np.zeros_like(self.arr(vel[k])) for k in ("u", "v", "w")}
        a3 = {k: self.arr(g3[k]) for k in ("u", "v", "w")}
        self._f("advect_velocity_adjoint")(W, H, D, _p(vel["u"]), _p(vel["v"]), _p(vel["w"]), _p(occ),
                                           C.byref(params), _p(a3["u"]), _p(a3["v"]),
                                           _p(a3["w"]), _p(g2["u"]), _p(g2["v"]), _p(g2["w"]))
        return g2

    def add_force_adjoint(self, W, H, D, vel, occ, params, g, gT, grho, gF=None):
        """In place on g (velocity); adds into gT, grho and gF (3, D, H, W) when given."""
        self._f("add_force_adjoint")(W, H, D, _p(vel["u"]), _p(vel["v"]), _p(vel["w"]), _p(occ), C.byref(params),
                                     _p(g["u"]), _p(g["v"]), _p(g["w"]), _p(gT), _p(grho), _p(gF))

    def step_adjoint(self, W, H, D, st, occ, params, F, g, gF):
        """Adjoint of one step(F) from state st; g (state adjoint) in place, gF += dL/dF."""
        Fa = None if F is None else self.arr(F)
        return self._f("step_adjoint")(W, H, D, _p(st["u"]), _p(st["v"]), _p(st["w"]), _p(st["T"]), _p(st["rho"]),
                                       _p(occ), C.byref(params), _p(Fa),
                                       _p(g["u"]), _p(g["v"]), _p(g["w"]), _p(g["T"]), _p(g["rho"]), _p(gF))

    def control_loss(self, W, H, D, st, occ, params, nsteps, F, target, grad=False):
        """L = sum (rho_n - target)^2 after nsteps steps with force F; with grad,
        also dL/dF (3, D, H, W) and the adjoint of the initial state."""
        loss = C.c_double(0.0)
        gF = np.zeros((3, D, H, W), self.dtype) if grad else None
        n0 = sum(st[k].size for k in ("u", "v", "w", "T", "rho"))
        g0 = np.zeros(n0, self.dtype) if grad else None
        s = {k: self.arr(st[k]) for k in ("u", "v", "w", "T", "rho")}
        Fa, ta = self.arr(F), self.arr(target)
        rc = self._f("control_loss")(W, H, D, _p(s["u"]), _p(s["v"]), _p(s["w"]),
                                     _p(s["T"]), _p(s["rho"]), _p(occ), C.byref(params),
                                     nsteps, _p(Fa), _p(ta), C.byref(loss), _p(gF), _p(g0))
        if rc != 0:
            raise RuntimeError(f"oracle control_loss failed: {rc}")
        return (loss.value, gF, g0) if grad else loss.value

    def state(self, wl):
        """Copy of a workload's state in this oracle's dtype."""
        return {k: self.arr(getattr(wl, k)).copy() for k in ("u", "v", "w", "T", "rho")}


def num_threads() -> int:
    return int(load().zqo_num_threads())
