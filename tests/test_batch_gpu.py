"""GPU: batched mixed-size stepping (zqs_batch_*) against one-at-a-time runs.

Each member of a batch must end in exactly the state zqs_grid_step leaves the
same grid in: the batched kernels run the single-grid tile functions on the
member's own buffers, so the comparison is bitwise (the 1e-5 relative L2
tolerance of the mixed-size configuration is asserted as well).
"""
import numpy as np
import pytest

from conftest import rel_l2
from zq_smokesimulation_gb300 import capi
from zq_smokesimulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu

FIELDS = ("u", "v", "w", "T", "rho")
TOL_BATCH = 1e-5


def make_grid(w, graph=True):
    g = capi.Grid(w.W, w.H, w.D)
    g.set_params(w.params)
    g.use_graph(graph)
    g.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
    return g


def assert_same(a: dict, b: dict, what: str):
    for k in FIELDS:
        assert a[k].shape == b[k].shape, (what, k)
        assert rel_l2(a[k], b[k]) <= TOL_BATCH, (what, k, rel_l2(a[k], b[k]))
        if not np.array_equal(a[k], b[k]):
            bad = np.argwhere(a[k] != b[k])
            raise AssertionError(f"{what} {k}: {len(bad)} mismatches, first {bad[:3].tolist()}")


def mixed_small(K=20):
    """Irregular small members: odd sizes, obstacles, one closed-solver member."""
    cases = [
        wl.small_case(24, 20, 16, seed=1, K=K, vel_amp=0.2),
        wl.small_case(17, 33, 9, seed=2, K=K, vel_amp=0.3),
        wl.small_case(32, 32, 32, seed=3, K=K, obstacle=False),
        wl.small_case(40, 24, 48, seed=4, K=K, closed=True, vel_amp=0.2),
        wl.small_case(9, 11, 7, seed=5, K=K),
        wl.small_case(66, 18, 30, seed=6, K=K, vel_amp=0.1),
    ]
    cases[1].params.step_time = 0.11
    cases[2].params.confine = 0.7
    cases[4].params.buoyancy = 2.0
    return cases


def run_single(cases, steps):
    out = []
    for w in cases:
        g = make_grid(w)
        g.step(steps)
        out.append(g.state())
        g.close()
    return out


@pytest.mark.parametrize("K", [20, 7, 0])
@pytest.mark.parametrize("graph", [True, False])
def test_batch_matches_single(zqs_lib, K, graph):
    cases = mixed_small(K)
    ref = run_single(cases, 3)
    grids = [make_grid(w) for w in cases]
    b = capi.Batch(grids)
    b.use_graph(graph)
    b.step(2)
    b.step(1)
    b.sync()
    for i, (g, r) in enumerate(zip(grids, ref)):
        assert_same(g.state(), r, f"member {i} K={K} graph={graph}")
    assert b.launch_count() > 0
    b.close()


def test_batch_more_members_than_one_advection_table(zqs_lib):
    """130 members: the advection kernels take their per-member parameters
    from by-value tables of at most 96 members, so this batch launches each
    advection stage as two chunks; every member still ends bit-identical to
    its own run."""
    rng = np.random.default_rng(5)
    cases = []
    for m in range(130):
        W, H, D = (int(x) for x in rng.integers(6, 15, size=3))
        w = wl.small_case(W, H, D, seed=100 + m, K=5, vel_amp=0.3, obstacle=bool(m % 3 == 0))
        w.params.step_time = float(rng.uniform(0.05, 0.2))
        cases.append(w)
    ref = run_single(cases, 2)
    grids = [make_grid(w) for w in cases]
    b = capi.Batch(grids)
    b.step(2)
    b.sync()
    for i, (g, r) in enumerate(zip(grids, ref)):
        assert_same(g.state(), r, f"member {i} of 130")
    b.close()
    for g in grids:
        g.close()


def test_batch_matches_oracle(zqs_lib, oracle32):
    cases = mixed_small(9)[:3]
    grids = [make_grid(w) for w in cases]
    b = capi.Batch(grids)
    b.step(2)
    b.sync()
    for w, g in zip(cases, grids):
        st = oracle32.state(w)
        rc, _ = oracle32.step(w.W, w.H, w.D, st, w.occ, w.params, 2)
        assert rc == 0
        out = g.state()
        for k in FIELDS:
            assert rel_l2(out[k], st[k]) <= TOL_BATCH, k
            assert np.array_equal(out[k], st[k]), (w.name, k)


def test_batch_sor_variants_equal(zqs_lib):
    cases = mixed_small(10)[:4]
    ref = run_single(cases, 2)
    batchable = []
    for i, v in enumerate(capi.sor_variants()):
        grids = [make_grid(w) for w in cases]
        b = capi.Batch(grids)
        try:
            b.set_sor_variant(i, 0)
        except capi.ZQSError as e:
            assert e.code == capi.ZQS_EUNSUPPORTED
            continue
        batchable.append(i)
        b.step(2)
        b.sync()
        for j, (g, r) in enumerate(zip(grids, ref)):
            assert_same(g.state(), r, f"variant {i} member {j}")
        # a forced z chunk splits columns into several chunks: same results
        grids2 = [make_grid(w) for w in cases]
        b2 = capi.Batch(grids2)
        b2.set_sor_variant(i, 5)
        b2.step(2)
        b2.sync()
        for j, (g, r) in enumerate(zip(grids2, ref)):
            assert_same(g.state(), r, f"variant {i} zchunk 5 member {j}")
    assert len(batchable) >= 4


def test_batch_picks_up_member_changes(zqs_lib):
    cases = mixed_small(12)[:3]
    # reference: member 1 changes dt after the first step, member 0 takes an
    # extra step of its own between the batch steps
    ref = []
    for i, w in enumerate(cases):
        g = make_grid(w)
        g.step(1)
        if i == 0:
            g.step(1)
        if i == 1:
            p = w.params.copy()
            p.step_time = 0.07
            g.set_params(p)
        g.step(1)
        ref.append(g.state())
        g.close()
    grids = [make_grid(w) for w in cases]
    b = capi.Batch(grids)
    b.step(1)
    b.sync()
    grids[0].step(1)
    grids[0].sync()
    p = cases[1].params.copy()
    p.step_time = 0.07
    grids[1].set_params(p)
    b.step(1)
    b.sync()
    for i, (g, r) in enumerate(zip(grids, ref)):
        assert_same(g.state(), r, f"member {i} after changes")


def test_batch_rejects_unsupported(zqs_lib):
    a = wl.small_case(16, 12, 10, K=10)
    c = wl.small_case(12, 12, 12, K=12)
    ga, gc = make_grid(a), make_grid(c)
    with pytest.raises(capi.ZQSError) as e:
        capi.Batch([ga, gc])            # different sor_iters
    assert e.value.code == capi.ZQS_EUNSUPPORTED
    with pytest.raises(capi.ZQSError) as e:
        capi.Batch([ga, ga])            # the same grid twice
    assert e.value.code == capi.ZQS_EINVAL
    r = wl.small_case(16, 12, 10, K=10, vel_mode=capi.ADV_VEL_INREG_OUTREG)
    gr = make_grid(r)
    with pytest.raises(capi.ZQSError) as e:
        capi.Batch([ga, gr])            # regular-grid advection has no batched form
    assert e.value.code == capi.ZQS_EUNSUPPORTED
    b = capi.Batch([ga])
    with pytest.raises(capi.ZQSError) as e:
        b.set_sor_variant(0, 0)         # shared-memory-only variants have no batched form
    assert e.value.code == capi.ZQS_EUNSUPPORTED
    with pytest.raises(capi.ZQSError) as e:
        b.set_sor_variant(999, 0)
    assert e.value.code == capi.ZQS_EINVAL
    fresh = capi.Grid(8, 8, 8)          # no parameters yet
    with pytest.raises(capi.ZQSError) as e:
        capi.Batch([fresh])
    assert e.value.code == capi.ZQS_ENOTREADY


@pytest.mark.slow
def test_batch64_matches_single(zqs_lib):
    """The 64-instance mixed-size configuration (K=200), 2 steps, every member."""
    cases = wl.batch_mixed(64)
    grids = [make_grid(w) for w in cases]
    b = capi.Batch(grids)
    b.step(2)
    b.sync()
    batched = [g.state() for g in grids]
    b.close()
    for g in grids:
        g.close()
    for i, w in enumerate(cases):
        g = make_grid(w)
        g.step(2)
        assert_same(batched[i], g.state(), f"batch64 member {i} {w.name}")
        g.close()
    assert float(sum(s["rho"].sum() for s in batched)) > 0.0
