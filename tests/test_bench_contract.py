"""CPU checks of bench.py's output contract: the reference arm (the oracle on
the host cores) prints one JSON line with the keys and units the GPU arm's
line carries, and its end-to-end entry moves no device bytes."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], capture_output=True, text=True,
                         cwd=ROOT, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    return json.loads(lines[0])


@pytest.mark.parametrize("config", ["pyramid", "batched"])
def test_reference_arm_prints_the_contract_line(config):
    steps = 2 if config == "pyramid" else 1
    d = _run("--impl", "reference", "--config", config, "--steps", str(steps), "--warmup", "1")
    assert d["impl"] == "reference"
    assert d["unit"] == "body-steps/s" and d["higher_is_better"] is True
    assert d["n_gpus"] == 1 and d["steps"] == steps and d["warmup"] == 1
    assert d["value"] > 0 and d["ms_per_step"] > 0
    assert d["metric"].startswith("body-steps/s")
    assert d["data"] == "synthetic" and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["unit"] == d["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    if config == "batched":
        assert d["config"]["bodies_per_gpu"] == 432126 and d["config"]["scenes_per_gpu"] == 1024
