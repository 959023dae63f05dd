"""CPU: bench.py's reference arm (the oracle port of the reference's numpy
sequence, timed on the host cores) prints one JSON line with the contract's
keys.  Runs a minimal sample on two processes."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    env = dict(os.environ)
    env["LP_BENCH_CPU_PROCS"] = "2"
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "2",
                        "--warmup", "3"], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["warmup"] >= 3 and line["value"] > 0 and line["higher_is_better"] is True
    assert line["steps"] == 2  # the requested steps are run
    sys.path.insert(0, ROOT)
    import bench
    assert line["config"] == bench.bench_config()  # the same config as the GPU arm
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == 2 and cb["value"] == line["value"]
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"],
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
