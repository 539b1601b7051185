"""The benchmark's reference arm runs on the host cores alone, so its JSON-line contract is checked
here without a GPU: one line with the metric, unit and config of the GB300 arm, the CPU baseline
block and an end-to-end block with no host-device traffic; under torchrun only rank 0 prints."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402  (module level defines constants only; nothing runs on import)


def run_reference(extra_env=None, n=512):
    env = dict(os.environ, OMP_NUM_THREADS="2")
    env.update(extra_env or {})
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "2",
                          "--warmup", "1", "--n", str(n)], capture_output=True, text=True, env=env, timeout=300)
    assert res.returncode == 0, res.stderr
    return [line for line in res.stdout.splitlines() if line.strip()]


def test_reference_arm_prints_one_contract_line():
    lines = run_reference()
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == "GFLOP/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["steps"] == 2 and d["warmup"] >= 3  # the warm-up is raised to at least 3 steps
    assert d["n_gpus"] == 1 and d["scaling"] == "weak" and d["vs_baseline"] is None
    assert d["dtype"] == "f64" and d["data"] == "synthetic"
    assert d["config"]["pattern"] == "star" and d["config"]["radius"] == 2 and d["config"]["n"] == 512
    assert "within L2" in d["config"]["l2"]  # 2 MB per array at n=512
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_print_nothing():
    lines = run_reference({"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"})
    assert lines == []
