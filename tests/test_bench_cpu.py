"""CPU: bench.py's reference arm (the reference algorithm timed on the host
cores, no GPU) keeps the JSON-line contract, on a small grid.

* one JSON line with impl, metric, unit, higher_is_better and a cpu_baseline
  describing the run;
* e2e equal to the line's value with no host<->device bytes;
* the per-iteration split into K*u, V-cycle and the rest adds up;
* under a launcher, ranks other than 0 print nothing and exit 0.
"""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0",
        "--size", "32", "16", "16", "--levels", "3", "--cpu-iters", "2"]


def _run(env_extra):
    env = dict(os.environ, OMP_NUM_THREADS="2", **env_extra)
    return subprocess.run(ARGS, capture_output=True, text=True, timeout=300, env=env, cwd=ROOT)


def test_reference_arm_line():
    out = _run({})
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    rec = json.loads(lines[0])
    assert rec["impl"] == "reference" and rec["unit"] == "s" and rec["higher_is_better"] is False
    assert rec["value"] > 0 and rec["steps"] == 1 and rec["config"]["grid"] == [32, 16, 16]
    cb = rec["cpu_baseline"]
    assert cb["value"] == rec["value"] and cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]
    e2e = rec["e2e"]
    assert e2e["value"] == rec["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    d = rec["detail"]
    assert abs(d["kbyu_s"] + d["vcycle_s"] + d["glue_s"] - d["iter_s"]) <= 1e-9 * max(d["iter_s"], 1.0)
    assert d["kbyu_s"] > 0 and d["vcycle_s"] > 0


def test_reference_arm_other_ranks_silent():
    out = _run({"RANK": "1", "WORLD_SIZE": "2"})
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.strip() == ""
