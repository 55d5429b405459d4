"""The benchmark's reference arm runs the oracle alone: its inputs come from
the oracle's restatement of the reference pre-processing, and the GPU
library is never loaded into the process."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_runs_without_the_gpu_library(oracle_built):
    env = dict(os.environ, OMP_NUM_THREADS="4")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "small",
                        "--steps", "1", "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT,
                       env=env)
    assert p.returncode == 0, p.stderr[-2000:]
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["config"]["gpu_library_loaded"] is False
    assert line["steps"] == 1 and line["warmup"] == 3
    assert line["value"] > 0 and line["cpu_baseline"]["single_core"]["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0
