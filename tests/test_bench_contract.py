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


def test_reference_arm_loads_no_project_library_and_shares_the_config():
    """The reference arm runs the reference's loops (restated in oracle/) on
    an instance generated in numpy: none of this project's libraries is
    loaded, and its config dict is the GPU arm's."""
    code = ("import runpy, sys, io, contextlib, json; sys.argv = ['bench.py', '--impl', 'reference', '--steps', '1', "
            "'--warmup', '1']; buf = io.StringIO()\n"
            "with contextlib.redirect_stdout(buf):\n"
            "    runpy.run_path('bench.py', run_name='__main__')\n"
            "maps = open('/proc/self/maps').read()\n"
            "print(json.dumps({'line': buf.getvalue(), 'help_libs': [l.split()[-1] for l in maps.splitlines() "
            "if 'libhelp_' in l]}))")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    out = json.loads(r.stdout.strip().splitlines()[-1])
    assert out["help_libs"] == []
    d = json.loads([ln for ln in out["line"].splitlines() if ln.startswith("{")][0])
    sys.path.insert(0, ROOT)
    import bench

    assert d["config"] == bench.bench_config(1)
