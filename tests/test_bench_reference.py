"""The reference arm of bench.py (`--impl reference`: the oracle port of the reference's CPU
path on the host cores) on a small node set: one JSON line with the contract's keys, the
same metric and workload naming as the GPU arm, and the CPU per-phase breakdown."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run(
        [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--nx", "48", "--steps", "1",
         "--warmup", "1", "--cpu-seconds", "1"],
        capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    import bench

    assert d["impl"] == "reference"
    assert d["metric"] == bench.METRIC and d["unit"] == "solves/s" and d["higher_is_better"] is True
    assert d["config"]["workload"] == bench.workload_name(48)
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 1
    assert d["e2e"] == {"value": d["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert cb["value_1_thread"] > 0 and cb["host_cores"] >= 1
    assert cb["cpu_model"] and "-O3" in cb["compiler_flags"] and "-march=native" not in cb["compiler_flags"]
    ph = cb["phases_ms_full_size"]
    for k in ("knn_all_nodes", "solves_all_nodes_extrapolated", "csc_build_per_op", "spmv_csc_1_thread",
              "spmv_rows_all_threads"):
        assert ph[k] > 0, k
