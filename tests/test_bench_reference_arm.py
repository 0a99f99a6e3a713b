"""bench.py's reference arm (the oracle port on the host cores) prints the
GPU arm's metric, unit and workload config with its own cpu_baseline and e2e
(CPU only)."""
import json
import os
import sys
import types

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line(capsys):
    sys.path.insert(0, ROOT)
    import bench
    specs = bench.ensemble_specs(256)[:6]
    bench.reference_arm(types.SimpleNamespace(steps=2, warmup=3), specs)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT and line["higher_is_better"] is True
    assert line["config"] == bench.workload_config(specs)
    assert line["steps"] == 2 and line["warmup"] == 3
    assert line["value"] > 0.0 and line["cpu_baseline"]["value"] == line["value"]
    assert line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"] == {"value": line["value"], "unit": bench.UNIT, "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
