"""CPU: bench.py's reference arm (the reference algorithm timed on the host
cores, no GPU) keeps the JSON-line contract, on a small grid.

* one JSON line with impl, metric, unit, higher_is_better and a cpu_baseline
  describing the run;
* e2e equal to the line's value with no host<->device bytes;
* the per-iteration split into K*u, V-cycle and the rest adds up;
* under a launcher, ranks other than 0 print nothing and exit 0;
* the GPU arm's roofline record (bytes and the FP32 dense-equivalent view) is
  consistent for a given launch time (a stand-in solver object, no GPU).
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


def test_roofline_record_consistent():
    sys.path.insert(0, ROOT)
    from sgldbench_gb300 import roofline as R

    class Stub:
        numNodes, numElements = 77105356, 75736061
        resY, resX, resZ = 512, 1024, 512

        def time_op(self, op, reps):
            assert op == "kbyu32" and reps == 20
            return 1.19

        def kbyu_tile(self):
            return {"tile_x": 8, "z_chunk": 24}

    rec = R.kbyu_f32_roofline(Stub(), reps=20)
    assert rec["bound"] == "hbm" and rec["unit"] == "GB/s"
    assert rec["algorithmic_bytes_per_launch"] == Stub.numNodes * 25 + Stub.numElements * 4
    assert abs(rec["achieved"] - rec["algorithmic_bytes_per_launch"] / 1.19e-3 / 1e9) <= 1e-6 * rec["achieved"]
    assert abs(rec["frac"] - rec["achieved"] / rec["peak"]) <= 1e-12
    assert rec["grid_nodes"] == 513 * 1025 * 513 and rec["traffic"] > rec["algorithmic_bytes_per_launch"]
    fp = rec["fp32_dense_equivalent"]
    assert fp["flops_per_element"] == 1176
    assert abs(fp["achieved_tflops"] - 1176 * Stub.numElements / 1.19e-3 / 1e12) <= 1e-9 * fp["achieved_tflops"]
    assert abs(fp["peak_tflops"] - 80.54784) <= 1e-6 and 0 < fp["frac"] < 1.5
    json.dumps(rec)
