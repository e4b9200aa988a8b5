"""bench.py's reference arm (the oracle port of the reference's CPU path on
the host cores) runs without a GPU and prints one JSON line with the keys
the benchmark contract asks for: the same metric and unit as the GPU arm,
"impl": "reference", an e2e entry with no host-device bytes and a
cpu_baseline describing the run."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    env = dict(os.environ, OMP_NUM_THREADS=str(min(8, os.cpu_count() or 1)))
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for k in ("metric", "unit", "value", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "config"):
        assert k in line, k
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert line["warmup"] >= 3  # at least three warm-up steps, whatever was asked
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["unit"] == line["unit"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == line["value"]
    assert "emax=6" in line["config"]["workload"]
