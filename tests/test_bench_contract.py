"""The benchmark's reference arm (CPU, the oracle restatement of the
reference) prints one JSON line with the contract's keys."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(*args):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), *args], cwd=ROOT,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    return json.loads(lines[0])


def test_reference_arm_line():
    d = _run("--impl", "reference", "--workload", "regular_2d", "--steps", "2", "--warmup", "3")
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference"
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 2
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("regular_2d") and d["config"]["n1"] == 257


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0 and not r.stdout.strip()


def test_both_arms_share_the_config():
    """The GPU arm's `config` is the same dict the reference arm prints
    (tank sizes the library derives go beside it, under `tank`)."""
    import tempfile
    sys.path.insert(0, ROOT)
    import bench
    with tempfile.TemporaryDirectory() as tmp:
        for name in bench.SINGLE_TANK:
            w = bench._single_tank(name, tmp)
            c = bench._workload_config(w)
            assert c["workload"].startswith(name) and c["n1"] == w["n1"] and c["n2"] == w["n2"]
    import inspect
    src = inspect.getsource(bench.run_cuda) + inspect.getsource(bench.run_reference)
    assert src.count('"config": _workload_config(w)') == 2
