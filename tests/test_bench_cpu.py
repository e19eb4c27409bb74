"""bench.py's reference arm runs on the CPU and prints one JSON line with the
keys the benchmark contract asks for (small workload)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_contract_line(covgpu, oracle):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0", "--N", "100", "--L", "120", "--nshuffle", "20", "--cpu-budget", "0.5"],
                       capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_extra_measurements_report_their_errors():
    """A failing extra measurement puts its error into the bench line instead
    of ending the run (the headline numbers are measured before the extras)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", os.path.join(ROOT, "bench.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)

    def bad(x):
        raise RuntimeError("covgpu error 90: %s" % x)

    assert b.guarded(lambda x, y=1: x + y, 2, y=3) == 5
    assert b.guarded(bad, "invalid argument") == {"error": "RuntimeError: covgpu error 90: invalid argument"}
