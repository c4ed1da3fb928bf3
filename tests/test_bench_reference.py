"""bench.py --impl reference (the CPU arm: the oracle port on the host cores) prints one JSON
line with the bench contract's keys; it runs without a GPU."""
import json
import os
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_json_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = [x for x in r.stdout.splitlines() if x.startswith("{")][-1]
    d = json.loads(line)
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["metric"] == "solves/s" and d["unit"] == "solves/s"
    assert d["value"] > 0 and d["higher_is_better"] is True
    assert d["config"]["unknowns"] == 30720 and "workload" in d["config"]
    cb = d["cpu_baseline"]
    assert cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_bench_precisions_are_the_library_constants():
    """bench.py's --precision names map to the C header's precision enum, and the default is the
    balanced mode (the fastest mode within the 1e-6 surface-current contract at C2)"""
    import importlib.util
    from beastgpu import lib as L
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    assert bench.PRECISIONS == {"mixed": L.MIXED, "mixed-accurate": L.MIXED_ACCURATE,
                                "mixed-balanced": L.MIXED_BALANCED, "fp64": L.FP64}
    sys_argv = sys.argv
    try:
        sys.argv = ["bench.py"]
        assert bench.parse().precision == "mixed-balanced"
    finally:
        sys.argv = sys_argv
