"""Failure detection without a GPU fault.

* A tensor-core block product whose producer issues nothing: the bounded
  mbarrier waits of k_subproj_tc give up, the kernel frees its tensor memory
  and sets the error flag, zqs_grid_synchronize reports ZQS_ETIMEOUT, and the
  next projection of the same grid runs normally.
* Device allocations made to fail on the host: the calls that make them return
  ZQS_ENOMEM, release what they had taken and leave the library usable.
"""
import ctypes as C

import numpy as np
import pytest

from zq_smokesimulation_gb300 import capi
from zq_smokesimulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

VEL = (capi.FIELD_U, capi.FIELD_V, capi.FIELD_W)


def _coarse_grid(w):
    g = capi.Grid(w.W, w.H, w.D)
    g.set_params(w.params)
    g.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
    return g


def test_tensor_core_wait_timeout_is_reported_and_recovers(zqs_lib):
    lib = zqs_lib
    w = wl.make("coarse64", K=20)
    ref = _coarse_grid(w)
    ref.project()
    ref.sync()
    want = [ref.download(f) for f in VEL]
    g = _coarse_grid(w)
    try:
        assert lib.zqs_debug_inject_tc_stall(1) == capi.ZQS_OK
        g.project()
    finally:
        lib.zqs_debug_inject_tc_stall(0)
    rc = lib.zqs_grid_synchronize(g.h, None)
    assert rc == capi.ZQS_ETIMEOUT, (rc, capi.last_error())
    assert "timed out" in capi.last_error()
    # the flag was consumed: the next synchronisation is clean
    assert lib.zqs_grid_synchronize(g.h, None) == capi.ZQS_OK
    # the context is usable and the same projection now matches the reference
    g.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
    g.project()
    assert lib.zqs_grid_synchronize(g.h, None) == capi.ZQS_OK
    for f, a in zip(VEL, want):
        assert np.array_equal(g.download(f), a), f
    g.close()
    ref.close()


def test_allocation_failures_return_enomem_and_release(zqs_lib):
    torch = pytest.importorskip("torch")
    lib = zqs_lib
    h = C.c_void_p()
    torch.cuda.synchronize()
    try:
        for nth in (0, 1):   # the grid's field block, then its dense occupancy
            assert lib.zqs_debug_fail_alloc(nth) == capi.ZQS_OK
            free0 = torch.cuda.mem_get_info()[0]
            rc = lib.zqs_grid_create(C.byref(h), 96, 80, 72)
            assert rc == capi.ZQS_ENOMEM, (nth, rc, capi.last_error())
            assert not h.value
            assert "cudaMalloc" in capi.last_error()
            torch.cuda.synchronize()
            assert torch.cuda.mem_get_info()[0] >= free0   # nothing kept
        lib.zqs_debug_fail_alloc(-1)
        # the library still works: a grid, an adjoint whose allocation fails, then one that does not
        w = wl.small_case(24, 20, 16, K=6)
        g = capi.Grid(w.W, w.H, w.D)
        g.set_params(w.params)
        g.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
        g.step(1)
        lib.zqs_debug_fail_alloc(0)
        with pytest.raises(capi.ZQSError) as e:
            capi.Adjoint(g, 4, 2)
        assert e.value.code == capi.ZQS_ENOMEM
        lib.zqs_debug_fail_alloc(-1)
        a = capi.Adjoint(g, 4, 2)
        a.close()
        # a batch whose table allocation fails
        g2 = capi.Grid(w.W, w.H, w.D)
        g2.set_params(w.params)
        g2.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
        lib.zqs_debug_fail_alloc(0)
        with pytest.raises(capi.ZQSError) as e:
            capi.Batch([g, g2])
        assert e.value.code == capi.ZQS_ENOMEM
        lib.zqs_debug_fail_alloc(-1)
        b = capi.Batch([g, g2])
        b.step(1)
        b.sync()
        b.close()
        g.step(1)
        g.close()
        g2.close()
    finally:
        lib.zqs_debug_fail_alloc(-1)


def test_fail_alloc_rejects_bad_arguments(zqs_lib):
    assert zqs_lib.zqs_debug_fail_alloc(-2) == capi.ZQS_EINVAL
    assert zqs_lib.zqs_debug_fail_alloc(-1) == capi.ZQS_OK
