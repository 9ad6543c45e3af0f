"""bench.py's reference arm on the CPU: one JSON line with the keys the bench
contract names, the same workload string as the GPU arm, and silence on
ranks other than 0 (replicas: rank 0 alone times the host code)."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)


def run(ranks=None, level=3):
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "LOCAL_RANK", "WORLD_SIZE")}
    env.update(ranks or {})
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--level", str(level), "--steps", "1",
                        "--warmup", "0"], cwd=REPO, capture_output=True, text=True, env=env, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    return [l for l in p.stdout.splitlines() if l.startswith("{")]


def test_reference_arm_line():
    import bench
    lines = run()
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "steps/s"
    assert d["higher_is_better"] is True and d["value"] > 0
    assert abs(d["ms_per_step"] - 1000.0 / d["value"]) < 1e-9 * d["ms_per_step"]
    assert d["config"]["workload"] == bench.workload(3)
    assert "642 points, 1280 triangles" in d["config"]["workload"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_silent():
    lines = run({"RANK": "1", "LOCAL_RANK": "1", "WORLD_SIZE": "2"})
    assert lines == []
