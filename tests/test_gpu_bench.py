"""bench.py runs end to end on a small droplet and prints one valid JSON line."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bench_small_json():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--small", "--steps", "10", "--warmup", "3",
                        "--plain-steps", "5", "--replicas", "4", "--requests", "3"],
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-3000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ["metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "roofline", "e2e", "clocks",
              "gpu_launches", "plain_fp64", "mixed_force_rms_rel_error"]:
        assert k in line, k
    assert line["value"] > 0 and line["e2e"]["value"] > 0
    assert line["mixed_force_rms_rel_error"] < 1e-5
    assert line["roofline"]["achieved"] and line["roofline"]["achieved"] > 0
    b = line["batched"]
    assert b["replicas"] == 4 and b["mixed"]["value"] > 0 and b["plain_fp64"]["value"] > 0
    sv = line["served"]
    assert sv["requests"] == 3 and 0 < sv["p50_latency_s"] <= sv["p99_latency_s"]
    assert sv["failed_requests"] == [] and sv["one_at_a_time_plain_fp64"]["atom_steps_per_s"] > 0
    sl = sv["slots_of_one_context"]
    assert sl["requests"] == 3 and sl["failed_requests"] == [] and sl["contexts_formed"] >= 1
    assert sv["arrival_limited"]["atom_steps_per_s"] > 0
    assert line["e2e_dropin_loop"]["value"] > 0
    assert line["cpu_baseline"]["value"] > 0 and line["force_rms_rel_error_vs_oracle"]["mixed"] < 1e-5
    assert line["force_rms_rel_error_vs_oracle"]["plain_fp64"] < 1e-10
    assert "measured" in line["roofline"]["peak_source"] and 0 < line["roofline"]["frac"] < 1.5


def test_bench_reference_arm_small():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--small", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
