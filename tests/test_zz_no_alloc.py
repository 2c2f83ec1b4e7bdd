"""The allocation-free projection entry point, zqs_project_sor_noalloc.

It serves callers that cannot allocate GPU memory while they project (a
pre-reserved memory pool, code running during a CUDA graph capture, runtimes
without an allocator): it works on the caller's device arrays with a fixed
working area built into the library.  This file is collected last so a run
that stops at the first failure has run every other test before it.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_l2
from zq_smokesimulation_gb300 import capi
from zq_smokesimulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def _reference_projection(lib, w, solver, K):
    """The existing (allocating) entry point on host copies of the same input."""
    out = {k: np.ascontiguousarray(getattr(w, k), np.float32).copy() for k in ("u", "v", "w")}
    occ = np.ascontiguousarray(w.occ, np.uint8)
    rc = lib.zqs_project_sor(out["u"].ctypes.data, out["v"].ctypes.data, out["w"].ctypes.data, occ.ctypes.data,
                             w.W, w.H, w.D, solver, K, C.c_float(1.9))
    assert rc == capi.ZQS_OK, capi.last_error()
    return out


def _noalloc(lib, dev, docc, w, solver, K):
    return lib.zqs_project_sor_noalloc(dev["u"].data_ptr(), dev["v"].data_ptr(), dev["w"].data_ptr(),
                                       docc.data_ptr(), w.W, w.H, w.D, solver, K, C.c_float(1.9), None)


def _device(torch, w):
    dev = {k: torch.from_numpy(np.ascontiguousarray(getattr(w, k), np.float32)).cuda() for k in ("u", "v", "w")}
    return dev, torch.from_numpy(np.ascontiguousarray(w.occ, np.uint8)).cuda()


def test_noalloc_projection_matches_allocating_entry_point(zqs_lib):
    torch = pytest.importorskip("torch")
    lib = zqs_lib
    K = 25
    # one-time setup first: a call with each solver type (kernel attributes,
    # the array's address and the kernels' loading happen on these)
    for closed in (False, True):
        w = wl.small_case(12, 10, 9, seed=3, K=3, closed=closed)
        dev, docc = _device(torch, w)
        assert _noalloc(lib, dev, docc, w, capi.SOLVER_CLOSED if closed else capi.SOLVER_OPEN, 3) == capi.ZQS_OK
    torch.cuda.synchronize()
    # two calls in a row on different grids: the second must not see the first's data
    cases = [((40, 33, 28), 11, False), ((64, 64, 64), 12, True)]
    for dims, seed, closed in cases:
        w = wl.small_case(*dims, seed=seed, K=K, vel_amp=0.3, closed=closed)
        solver = capi.SOLVER_CLOSED if closed else capi.SOLVER_OPEN
        ref = _reference_projection(lib, w, solver, K)
        dev, docc = _device(torch, w)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        assert _noalloc(lib, dev, docc, w, solver, K) == capi.ZQS_OK, capi.last_error()
        torch.cuda.synchronize()
        # after the setup calls, a call takes no device memory
        assert torch.cuda.mem_get_info()[0] == free_before
        for k in ("u", "v", "w"):
            got = dev[k].cpu().numpy()
            assert rel_l2(got, ref[k]) <= 1e-5, k
            assert np.array_equal(got, ref[k]), k


def test_noalloc_rejects_grids_beyond_its_fixed_area(zqs_lib):
    torch = pytest.importorskip("torch")
    t = torch.zeros(8, device="cuda")
    rc = zqs_lib.zqs_project_sor_noalloc(t.data_ptr(), t.data_ptr(), t.data_ptr(), t.data_ptr(), 80, 80, 80,
                                         capi.SOLVER_OPEN, 5, C.c_float(1.0), None)
    assert rc == capi.ZQS_EINVAL
    assert "fixed working area" in capi.last_error()
