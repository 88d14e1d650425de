"""bench.py's reference arm runs on the host cores alone: rank 0 prints one
JSON line with the contract's keys, on the headline's metric and workload;
other ranks print nothing and exit 0.  The ncu summaries under profiles/
give commands that run committed files with the clocks left unlocked."""
import json
import os
import re
import subprocess
import sys

from conftest import ROOT

ARGS = [sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3", "--cpu-paths", "2048"]
KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e")


def _run(env=None):
    r = subprocess.run(ARGS, cwd=ROOT, capture_output=True, text=True, timeout=600, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    return [ln for ln in r.stdout.splitlines() if ln.startswith("{")]


def test_reference_arm_line():
    lines = _run()
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in KEYS:
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["unit"] == "path-steps/s" and d["e2e"]["value"] == d["value"]
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == d["value"] and cb["cores"] >= 1 and "2048 paths" in cb["sample"]
    sys.path.insert(0, ROOT)
    import bench
    assert d["metric"] == bench.METRIC and d["config"]["workload"] == bench.WORKLOAD


def test_reference_arm_other_ranks_print_nothing():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    assert _run(env) == []


def test_profile_summaries_cite_committed_commands():
    """Each ncu summary gives the command that made it: every ncu line keeps
    the clocks unlocked, and every script it runs is a committed file."""
    d = os.path.join(ROOT, "profiles")
    names = sorted(n for n in os.listdir(d) if n.endswith((".md", ".txt")))
    assert names
    for n in names:
        with open(os.path.join(d, n)) as f:
            text = f.read()
        ncu = [ln for ln in text.splitlines() if re.match(r"\s*ncu ", ln)]
        assert ncu, n
        assert all("--clock-control none" in ln for ln in ncu), n
        for script in set(re.findall(r"python ([\w/.-]+\.py)", text)):
            assert os.path.isfile(os.path.join(ROOT, script)) and not script.startswith("_work"), (n, script)


def test_equal_rmse_speedup_model():
    """RMSE^2 = se^2 N/N' + bias^2: FP32 matches the FP64 RMSE at N with
    N' = N se^2 / (se^2 - bias^2) paths, so the time ratio is
    (thr32 / thr64)(1 - bias^2 / se^2); 0 once the bias alone reaches se."""
    sys.path.insert(0, ROOT)
    import bench
    assert bench.equal_rmse_speedup(100.0, 1.0, 0.0, 0.5) == 100.0
    assert abs(bench.equal_rmse_speedup(100.0, 1.0, 0.25, 0.5) - 75.0) < 1e-12
    assert bench.equal_rmse_speedup(100.0, 1.0, 0.5, 0.5) == 0.0
    assert bench.equal_rmse_speedup(100.0, 1.0, 0.1, 0.0) is None
