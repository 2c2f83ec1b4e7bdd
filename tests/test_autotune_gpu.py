"""The SOR autotuner: temporal_depth 0 runs the variant and z chunk measured
fastest for the grid's shape on this device, chosen once per (device, shape)
and kept in memory and in the file named by ZQS_TUNE_CACHE.  Every variant is
bit-identical to one-colour sweeps, so the choice never changes results."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from zq_smokesimulation_gb300 import capi
from zq_smokesimulation_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]


def _grid(w, depth):
    g = capi.Grid(w.W, w.H, w.D)
    g.set_params(w.params)
    g.set_sor_config(depth, False)
    g.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
    return g


def test_tuned_choice_is_bit_identical_and_cached(zqs_lib, tmp_path, monkeypatch):
    cache = tmp_path / "tune.txt"
    monkeypatch.setenv("ZQS_TUNE_CACHE", str(cache))
    monkeypatch.delenv("ZQS_AUTOTUNE", raising=False)
    w = wl.small_case(72, 40, 52, K=9, vel_amp=0.3)   # a shape no other test tunes
    g = _grid(w, 0)
    v, zc, us = g.sor_choice()
    info = capi.sor_variants()
    assert 0 <= v < len(info) and info[v].ctas_per_sm >= 1 and zc >= 1 and us > 0.0
    g.step(2)
    ref = _grid(w, 1)
    ref.set_sor_config(1, True)  # one launch per colour
    ref.step(2)
    for f in (capi.FIELD_U, capi.FIELD_V, capi.FIELD_W, capi.FIELD_DENSITY, capi.FIELD_PRESSURE):
        assert np.array_equal(g.download(f), ref.download(f)), f
    lines = cache.read_text().splitlines()
    assert any("|72x40x52|" in ln and ln.split()[1] == str(v) for ln in lines)
    # a second grid of the shape takes the choice without measuring again
    g2 = _grid(w, 0)
    assert g2.sor_choice()[:2] == (v, zc)
    # a new process reads it from the file
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from zq_smokesimulation_gb300 import capi, workloads as wl\n"
            "w = wl.small_case(72, 40, 52, K=9, vel_amp=0.3)\n"
            "g = capi.Grid(w.W, w.H, w.D); g.set_params(w.params); g.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)\n"
            "print(*g.sor_choice()[:2])\n" % str(ROOT))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300,
                         env=dict(os.environ, ZQS_TUNE_CACHE=str(cache)))
    assert out.returncode == 0, out.stderr
    assert out.stdout.split()[-2:] == [str(v), str(zc)]
    assert len(cache.read_text().splitlines()) == len(lines)   # nothing measured, nothing appended
    for x in (g, g2, ref):
        x.close()


def test_explicit_depth_and_disabled_tuner_keep_the_default(zqs_lib, monkeypatch):
    w = wl.small_case(20, 18, 16, K=4)
    g = _grid(w, 2)
    assert g.sor_choice()[0] == -1 or capi.sor_variants()[g.sor_choice()[0]].depth == 2
    monkeypatch.setenv("ZQS_AUTOTUNE", "0")
    g0 = _grid(wl.small_case(22, 18, 16, K=4), 0)
    v, zc, us = g0.sor_choice()
    assert us == 0.0   # nothing measured
    g0.step(1)
    g.close()
    g0.close()
