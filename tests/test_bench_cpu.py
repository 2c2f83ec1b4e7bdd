"""bench.py's reference arm on CPU: the FP32 oracle timed on the host cores on
the bench's own configuration (one full step per timed step), printed as one
JSON line with the same metric, unit and workload keys as the GPU arm (no GPU
needed)."""
import argparse
import json

import pytest


def test_reference_arm_prints_one_contract_line(capsys, monkeypatch):
    pytest.importorskip("oracle.binding").load()
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    import bench
    args = argparse.Namespace(workload="plain64", cpu_sample="", steps=2, warmup=3, gpus=1)
    bench.run_reference(args)
    lines = [ln for ln in capsys.readouterr().out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["steps"] == 2 and d["warmup"] == 3 and d["n_gpus"] == 1 and d["higher_is_better"] is True
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"] and d["e2e"]["value"] == d["value"]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["cpu_model"] and d["cpu_baseline"]["grid"] == [64, 64, 64]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    cfg = d["config"]
    assert cfg["workload"] == "plain64" and cfg["grid"] == [64, 64, 64]
    assert cfg["sor_iters"] == 200 and cfg["substeps"] == 20


def test_sor_traffic_read_per_variant():
    """The roofline's `traffic` comes from the committed ncu summary of the SOR
    pass, one `sor_variant` / `traffic_bytes_per_launch` pair per captured
    variant; a variant that was not captured reports None."""
    import bench
    for v in (18, 25, 26):   # the fixed default and the tuner's usual picks at 256^3
        t = bench.profile_traffic("k_sor_plain256", v)
        assert t is not None and 1.5e8 < t < 2.5e8, (v, t)
    assert bench.profile_traffic("k_sor_plain256", 999) is None
    assert bench.profile_traffic("no_such_profile", 18) is None
