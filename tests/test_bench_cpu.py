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
