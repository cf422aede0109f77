"""The reference arm of bench.py (the C/OpenMP restatement of the reference
step on the host cores) on a small grid: one JSON line with the contract's
keys, the requested warm-up, and nothing from ranks other than 0."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(env_extra, gpus=1, rc=0):
    env = dict(os.environ, **env_extra)
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--n", "64", "--steps", "2",
                        "--warmup", "3", "--gpus", str(gpus)], cwd=ROOT, env=env, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == rc, r.stderr[-2000:]
    return [l for l in r.stdout.splitlines() if l.startswith("{")]


def test_reference_arm_line():
    lines = _run({})
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 3
    assert d["higher_is_better"] is True and d["dtype"] == "f64"
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_are_silent():
    assert _run({"RANK": "1", "WORLD_SIZE": "2"}, gpus=2) == []


def test_gpus_must_match_the_launched_world():
    """--gpus N under a launcher whose WORLD_SIZE differs is an error, not a
    silent single-GPU run."""
    assert _run({"RANK": "0", "WORLD_SIZE": "1"}, gpus=2, rc=2) == []


def test_both_arms_share_one_config():
    sys.path.insert(0, ROOT)
    import bench
    lines = _run({})
    d = json.loads(lines[0])
    assert d["config"] == bench.bench_config(64, 1)
