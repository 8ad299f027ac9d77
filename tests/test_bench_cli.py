"""CPU checks of bench.py's command line and of the reference arm's JSON line.

The reference arm runs the C oracle on the host cores, so its line can be
checked here without a GPU: one JSON object with the metric, unit, config and
the reference-arm keys (impl, cpu_baseline, e2e with zero copy bytes).
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e", "impl"}


def _run(*argv, timeout=240):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *argv], cwd=ROOT, capture_output=True,
                       text=True, timeout=timeout)
    return r


def _line(r):
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, r.stdout
    return json.loads(lines[0])


def test_reference_arm_plain_line():
    d = _line(_run("--impl", "reference", "--n", "20", "--steps", "1", "--warmup", "1", "--cpu-seconds", "1"))
    assert KEYS <= set(d), KEYS - set(d)
    assert d["impl"] == "reference" and d["unit"] == "perm/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "perm/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("plain permanent, top-left 20x20 block")


def test_reference_arm_batched_config_names_the_batch():
    d = _line(_run("--impl", "reference", "--workload", "batched", "--batch-count", "32", "--batch-kmax", "14",
                   "--steps", "1", "--warmup", "1"))
    assert KEYS <= set(d)
    assert d["config"]["workload"].startswith("32 uneven k x k permanents, k uniform 8..14")
    assert d["cpu_baseline"]["kind"] == "port" and "32-instance batch" in d["cpu_baseline"]["sample"]


@pytest.mark.parametrize("argv", [["--batch-count", "0"], ["--batch-kmax", "7"], ["--batch-kmax", "33"]])
def test_batch_options_are_checked(argv):
    r = _run("--impl", "reference", "--workload", "batched", *argv, timeout=60)
    assert r.returncode == 2 and "--batch-kmax in 8..32" in r.stderr
