"""CPU: bench.py's reference arm (the reference's CPU algorithm on the host's cores) keeps the
bench line's contract on a small workload, and ranks other than 0 print nothing."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SMALL = ["--impl", "reference", "--n", "3000", "--dim", "48", "--clusters", "16", "--queries", "64",
         "--batch", "4", "--steps", "5", "--warmup", "3"]


def _run(extra_env=None):
    env = dict(os.environ)
    env.update(extra_env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py")] + SMALL, cwd=ROOT, env=env,
                          capture_output=True, text=True, timeout=300)


def test_reference_arm_line():
    p = _run()
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [l for l in p.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["metric"] == "exact top-10 QPS at 3Kx48" and d["unit"] == "queries/s"
    assert d["value"] > 0 and d["steps"] == 5 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["higher_is_better"] is True and d["vs_baseline"] is None
    assert d["config"]["batch"] == 4 and d["config"]["n"] == 3000 and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == d["value"] and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "queries/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}


def test_reference_arm_other_ranks_are_silent():
    p = _run({"RANK": "1"})
    assert p.returncode == 0, p.stderr[-2000:]
    assert p.stdout.strip() == ""
