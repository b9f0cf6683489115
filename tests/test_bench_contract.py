"""The benchmark's JSON line on the CPU: the reference arm (the oracle on the
host cores) on the small closed-basin workload prints one line with the
fields the benchmark contract names, and the helpers the GPU arm's
roofline uses read the committed ncu summaries."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "c0",
                          "--steps", "2", "--warmup", "3"], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] == 3
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert "257x193" in d["config"]["workload"]


def test_profile_traffic_keys():
    sys.path.insert(0, ROOT)
    import bench

    # the headline form and its side forms quote the DRAM traffic of their captures
    for form in ("mixed", "mixed-fp32prep", "mixed-fct4", "mixed-mpdata", "mixed-diff"):
        t = bench.profile_traffic(f"{bench.TRAFFIC_KEY[form]}_c1")
        assert t is not None and 1e10 < t < 1e11, (form, t)
    assert bench.profile_traffic("no_such_kernel_c1") is None
