"""The reference arm of bench.py on the CPU: one JSON line with the
contract's keys, whole ICs of the oracle port timed one per step (a small
grid and PLT mesh here so the test is quick)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--ref-ngrid", "32", "--ref-plt-ngrid", "16",
                        "--steps", "2", "--warmup", "1"], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["steps"] == 2 and d["warmup"] == 1 and d["value"] > 0
    assert d["unit"] == "particles/s" and d["higher_is_better"] is True
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert "2x512^3" in d["config"]["workload"] and d["config"]["reference_sample"] == "2x32^3 per step"
    assert "2 whole 3LPT+PLT BCC 2x32^3 ICs" in d["cpu_baseline"]["sample"]
    # the line's time is the timed whole ICs themselves: steps x ms_per_step = their sum
    assert abs(d["value"] - 2 * 32 ** 3 / (d["ms_per_step"] / 1e3)) < 1e-6 * d["value"]
