"""bench.py's reference arm on the CPU: one JSON line with the contract's
keys, the metric and config of the GPU arm, the CPU baseline describing the
run, and an end-to-end entry that moves no bytes."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "1"], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e", "impl"):
        assert key in d, key
    assert d["impl"] == "reference" and d["unit"] == "GB/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["warmup"] == 1
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0
    assert "workload" in d["config"]


def test_presolve_entry():
    """The bench line's presolve entry (host code, timed on the host CPU):
    eight rows off the ungrounded flow, not applicable to config 1."""
    sys.path.insert(0, ROOT)
    import bench

    d = bench.presolve_time()
    json.dumps(d)
    assert d["mcf_200x200x8_ungrounded"]["rows_removed"] == 8
    assert d["mcf_200x200x8_ungrounded"]["rows"] == 479200
    assert d["config1_random"]["result"].startswith("not applicable")
    assert d["mcf_200x200x8_ungrounded"]["s"] > 0 and d["config1_random"]["s"] > 0
