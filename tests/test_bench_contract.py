"""bench.py's reference arm (CPU only): the JSON line the benchmark contract
asks for, on the small arc workload so that it runs in seconds."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    """Each step is one timed LM iteration of a whole-scene CPU solve: with
    more steps than one solve's iterations, a new solve starts, and the line
    reports exactly the steps it timed."""
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "arc", "--steps", "13",
                        "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads([l for l in r.stdout.splitlines() if l.startswith("{")][-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["value"] > 0 and line["unit"] == "LM iters/s"
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] in ("reference", "port") and line["cpu_baseline"]["cores"] >= 1
    assert "workload" in line["config"] and line["config"]["iterations"] == 10
    assert line["steps"] == 13 and line["warmup"] == 3
    per = line["seconds_per_iteration"]
    assert 0 < per["min"] <= per["median"] <= per["max"]
    assert abs(line["value"] * line["ms_per_step"] * 1e-3 - 1.0) < 1e-9
    assert "from 2 solve(s)" in line["cpu_baseline"]["sample"]


def test_reference_arm_two_ranks():
    """Launched as the driver launches N > 1 (torchrun, 127.0.0.1): rank 0
    alone prints the line, the other rank exits 0 without work."""
    # --standalone picks its own free rendezvous port on 127.0.0.1
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--standalone", "--local-addr", "127.0.0.1",
                        "--nnodes=1", "--nproc-per-node", "2", "bench.py", "--impl", "reference", "--workload", "arc",
                        "--steps", "1", "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1 and json.loads(lines[0])["impl"] == "reference"
