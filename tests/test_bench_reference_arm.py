"""The reference arm of bench.py (`--impl reference`): the reference
algorithm on the host cores for the bench workload, K timed iterations after
W warm-up ones, one JSON line from rank 0 with the CPU baseline and a
host-only e2e record; other ranks print nothing."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(env_extra, *args):
    env = dict(os.environ, **env_extra)
    return subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", *args],
                          cwd=REPO, env=env, capture_output=True, text=True, timeout=600)


def test_reference_arm_times_k_iterations_and_prints_one_line():
    p = _run({}, "--steps", "1", "--warmup", "1")
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["steps"] == 1 and d["warmup"] == 1 and "requested_steps" not in d
    assert d["unit"] == "iter/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and abs(d["ms_per_step"] - 1000.0 / d["value"]) < 1e-6 * d["ms_per_step"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert "reference basis" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["grid"] == 54 and d["config"]["l_max"] == 5


def test_reference_arm_other_ranks_are_silent():
    p = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, "--steps", "1", "--warmup", "1")
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""
