"""Seeded input generation and occupancy builders (no GPU)."""
import numpy as np

from zq_smokesimulation_gb300 import capi
from zq_smokesimulation_gb300 import workloads as wl


def test_splitmix64_known_values():
    # SplitMix64 of state seed + n*golden (n = 1, 2, 3) for seed 0
    z = wl.splitmix64(0, 3)
    assert [int(x) for x in z] == [0xE220A8397B1DCDAF, 0x6E789E6AA1B965F4, 0x06C45D188009454F]


def test_uniform_range_and_determinism():
    a = wl.uniform(5, 10000, -1e-3, 1e-3)
    b = wl.uniform(5, 10000, -1e-3, 1e-3)
    assert a.dtype == np.float32 and np.array_equal(a, b)
    assert a.min() >= -1e-3 and a.max() < 1e-3
    assert abs(float(a.mean())) < 5e-5


def test_walls_and_obstacle():
    occ = wl.walls_open_top(8, 8, 8)
    assert occ[1:7, 7, 1:7].sum() == 0       # open top row stays free inside the side walls
    assert occ[:, 0, :].all() and occ[0].all() and occ[7].all() and occ[:, :, 0].all() and occ[:, :, 7].all()
    wl.add_box(occ, 2, 3, 2, 4, 3, 3)
    assert occ[3, 2:5, 2:4].all() and occ[3].sum() == 22 + 6   # side walls + bottom of an inner plane, box


def test_live_faces_open_rule():
    occ = np.zeros((3, 3, 3), np.uint8)
    occ[1, 1, 1] = 1
    lu, lv, lw = wl.live_faces(occ)
    assert not lu[1, 1, 1] and not lu[1, 1, 2] and lu[1, 1, 0] and lu[1, 1, 3]
    assert lv[1, 0, 1] and not lv[1, 1, 1] and not lv[1, 2, 1] and lv[1, 3, 1]
    assert lw.sum() == 4 * 9 - 2


def test_baseline_workloads_shapes():
    w = wl.make("plain64")
    assert (w.W, w.params.sor_iters, w.steps, w.params.n_sources) == (64, 200, 100, 1)
    assert w.params.sources[0].shape == capi.SOURCE_SPHERE and w.params.sources[0].hx == 6.0
    assert abs(float(w.params.omega) - 1.9) < 1e-6 and abs(float(w.params.vel_atten) - 0.99) < 1e-6
    lu, lv, lw = wl.live_faces(w.occ)
    assert np.all(w.u[~lu] == 0) and np.abs(w.u).max() <= 1e-3 and np.abs(w.u[lu]).max() > 9e-4
    w = wl.make("plain128_obs", K=4)
    assert w.occ[48:81, 56:73, 48:81].all() and w.params.sor_iters == 4
    w = wl.make("plain256", K=1)
    assert w.params.n_sources == 4
    for q in range(4):
        s = w.params.sources[q]
        assert 8 <= s.hx <= 16 and s.cy <= 25.6 and 0.5 <= s.density <= 1 and 0.5 <= s.temperature <= 1
