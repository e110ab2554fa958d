"""The reference arm of bench.py (`--impl reference`): the reference
algorithm on the host cores for the bench workload, K timed iterations after
W warm-up ones, one JSON line from rank 0 with the CPU baseline and a
host-only e2e record; other ranks print nothing.  Also the algorithmic bytes
per launch that the GPU arm's roofline divides by."""
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
    assert 0 < cb["one_thread_value"]
    assert d["e2e"] == {"value": d["value"], "unit": "iter/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["grid"] == 54 and d["config"]["l_max"] == 5


def test_reference_arm_other_ranks_are_silent():
    p = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}, "--steps", "1", "--warmup", "1")
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""


def test_algorithmic_bytes_of_the_iteration_kernels():
    """Per-launch algorithmic bytes the roofline divides by, at 54^3 odd
    l <= 5 (N = 157,464 points, 21 functions, D = 3,306,744): x/y kinetic 16 B,
    z kinetic 24 B and update 24 B per coefficient; potential stream 231 FP32
    block entries per point plus 32 B per coefficient; 463 MB per iteration."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_for_bytes", os.path.join(REPO, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    N, nn = 54 ** 3, 21
    D = N * nn
    assert D == 3306744
    sb = bench.stage_bytes(bench._load("bsl_inputs_b", os.path.join(bench.PKG, "inputs.py")).CONFIG_METRIC, D, N,
                           nn, True)
    assert [round(x / 1e5) / 10 for x in sb] == [52.9, 79.4, 251.3, 79.4]
    assert abs(sum(sb) - 462944184) <= 8
